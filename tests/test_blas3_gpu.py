"""SYRK / SYMM / TRSM on the GPU against host BLAS (scipy.linalg.blas: the
OpenBLAS calls the reference's DeviceOpenBLAS makes), f64 within 1e-12 and f32
within 1e-5 relative Frobenius error; the triangle SYRK does not write and the
triangle SYMM does not read are checked to stay untouched / unused."""

import numpy as np
import pytest

import rstsr_gb300 as rt
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu
sblas = pytest.importorskip("scipy.linalg.blas")

TOL = {np.float64: 1e-12, np.float32: 1e-5}


def dev_matrix(x, dev, order):
    x = np.ascontiguousarray(x) if order == "C" else np.asfortranarray(x)
    st = (x.shape[1], 1) if order == "C" else (1, x.shape[0])
    return rt.from_host_layout(x.ravel(order=order), x.shape, st, 0, dev)


def blas(dtype, name):
    return getattr(sblas, ("d" if dtype == np.float64 else "s") + name)


@pytest.mark.parametrize("order", ["C", "F"])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("beta", [0.0, 0.5])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_syrk(dev, order, uplo, trans, beta, dtype):
    rng = np.random.default_rng(1)
    n, k = 150, 70
    a = rng.standard_normal((n, k) if trans == "N" else (k, n)).astype(dtype)
    c0 = rng.standard_normal((n, n)).astype(dtype)
    ta, tc = dev_matrix(a, dev, order), dev_matrix(c0, dev, order)
    rt.syrk(ta, tc, uplo, trans, alpha=1.5, beta=beta)
    got = tc.to_numpy()
    want = blas(dtype, "syrk")(1.5, a, beta=beta, c=np.asfortranarray(c0), trans=0 if trans == "N" else 1,
                               lower=1 if uplo == "L" else 0)
    tri = np.tril if uplo == "L" else np.triu
    other = np.triu if uplo == "L" else np.tril
    assert rel_err(tri(got), tri(want)) <= TOL[dtype]
    np.testing.assert_array_equal(other(got, 1 if uplo == "L" else -1), other(c0, 1 if uplo == "L" else -1))


@pytest.mark.parametrize("order", ["C", "F"])
@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_symm(dev, order, side, uplo, dtype):
    rng = np.random.default_rng(2)
    m, n = 120, 90
    na = m if side == "L" else n
    s = rng.standard_normal((na, na)).astype(dtype)
    s = (s + s.T) / 2
    a = s.copy()
    junk = np.triu_indices(na, 1) if uplo == "L" else np.tril_indices(na, -1)
    a[junk] = np.nan  # the triangle SYMM must not read
    b = rng.standard_normal((m, n)).astype(dtype)
    c0 = rng.standard_normal((m, n)).astype(dtype)
    ta, tb, tc = dev_matrix(a, dev, order), dev_matrix(b, dev, order), dev_matrix(c0, dev, order)
    rt.symm(ta, tb, tc, side, uplo, alpha=0.75, beta=-1.25)
    want = 0.75 * (s @ b if side == "L" else b @ s) - 1.25 * c0.astype(np.float64)
    assert rel_err(tc.to_numpy(), want) <= TOL[dtype]


@pytest.mark.parametrize("order", ["C", "F"])
@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("transa", ["N", "T"])
@pytest.mark.parametrize("diag", ["N", "U"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_trsm(dev, order, side, uplo, transa, diag, dtype):
    rng = np.random.default_rng(3)
    m, n = 200, 70  # four row blocks of 64, the last one partial
    na = m if side == "L" else n
    a = rng.standard_normal((na, na)) * 0.1 + np.eye(na) * 2.0
    a = (np.tril(a) if uplo == "L" else np.triu(a)).astype(dtype)
    if diag == "U":
        np.fill_diagonal(a, 7.0)  # not read
    b = rng.standard_normal((m, n)).astype(dtype)
    ta, tb = dev_matrix(a, dev, order), dev_matrix(b, dev, order)
    rt.trsm(ta, tb, side, uplo, transa, diag, alpha=2.0)
    want = blas(dtype, "trsm")(2.0, a, b, side=0 if side == "L" else 1, lower=1 if uplo == "L" else 0,
                               trans_a=0 if transa == "N" else 1, diag=0 if diag == "N" else 1)
    assert rel_err(tb.to_numpy(), want) <= TOL[dtype] * (10 if dtype == np.float32 else 1)


def test_trsm_large_property(dev):
    """A 2048 x 2048 lower system with 512 right-hand sides: op(A) X reproduces B."""
    rng = np.random.default_rng(4)
    n, r = 2048, 512
    a = np.tril(rng.standard_normal((n, n)) * 0.02) + np.eye(n) * 2.0
    b = rng.standard_normal((n, r))
    ta, tb = rt.asarray(a, dev), rt.asarray(b, dev)
    x = rt.trsm(ta, tb, "L", "L", "N", "N").to_numpy()
    assert rel_err(a @ x, b) <= 1e-12
