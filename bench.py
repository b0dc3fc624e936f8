"""Benchmark of the GB300 device backend on the memory-bound strided workload.

Workload (one "step"): for f64, f32 and i32 tensors of shape [32,64,128,128]
in four input layouts (C-contiguous, F-contiguous, axis-permuted view,
step-2 innermost slice), run the four hot-path operations of the rstsr
tensor layer through the C ABI:
  1. permute_dims(0,2,1,3) + to_contig (C order)   assign_arbitrary
  2. a * b + c with c of shape [1,64,1,128]         fused one-pass kernel
  3. sum over axes (1, 3)                           reduce_axes
  4. argmax over the last axis                      argreduce_axes
Inputs are seeded synthetic data (uniform(-1,1), i32 uniform in [-1000,1000])
resident in HBM; every tensor is larger than the 129 MB L2 on its own.

Metric: algorithmic HBM GB/s over the whole step (bytes the operations must
move, counted per element of the logical tensors), the device-timed `value`;
`e2e` repeats the step with the inputs copied from pinned host memory and the
results copied back inside the timed region.

`--impl reference` times the reference's CPU algorithm (the OpenMP
restatement of rstsr's rayon kernels in oracle/) on the host cores.
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from rstsr_gb300 import replicas  # noqa: E402

SHAPE = (32, 64, 128, 128)
CSHAPE = (1, 64, 1, 128)
N = int(np.prod(SHAPE))
DTYPES = [("f64", np.float64), ("f32", np.float32), ("i32", np.int32)]
LAYOUTS = ["c", "f", "perm", "slice"]
METRIC = "f64 GEMM TFLOP/s Ozaki-split vs native FP64 at ≤1e-12 rel err; elementwise HBM GB/s"
WORKLOAD = ("strided ops [32,64,128,128] x {f64,f32,i32} x {C,F,permuted,step-2 slice}: "
            "permute(0,2,1,3)+to_contig, a*b+c (c [1,64,1,128]), sum(1,3), argmax(-1)")


def c_stride(shape):
    st, acc = [], 1
    for d in reversed(shape):
        st.append(acc)
        acc *= max(d, 1)
    return tuple(reversed(st))


def f_stride(shape):
    st, acc = [], 1
    for d in shape:
        st.append(acc)
        acc *= max(d, 1)
    return tuple(st)


def layout_of(kind, shape):
    """(base buffer length, view strides, offset) of one input layout."""
    n = int(np.prod(shape))
    if kind == "c":
        return n, c_stride(shape), 0
    if kind == "f":
        return n, f_stride(shape), 0
    if kind == "perm":
        base = (shape[0], shape[2], shape[1], shape[3])
        st = list(c_stride(base))
        st[1], st[2] = st[2], st[1]
        return n, tuple(st), 0
    if kind == "slice":
        base = tuple(shape[:-1]) + (shape[-1] * 2,)
        st = list(c_stride(base))
        st[-1] *= 2
        return 2 * n, tuple(st), 0
    raise ValueError(kind)


def host_data(dt, n, seed):
    rng = np.random.default_rng(seed)
    if np.dtype(dt).kind == "f":
        return rng.uniform(-1.0, 1.0, n).astype(dt)
    return rng.integers(-1000, 1001, n).astype(dt)


def permuted_view(shape, stride):
    ax = (0, 2, 1, 3)
    return tuple(shape[a] for a in ax), tuple(stride[a] for a in ax)


def op_bytes(esize, kind):
    """Algorithmic bytes of each operation (logical elements only)."""
    copy_needed = kind != "perm"  # the permuted view of 'perm' is already C-contiguous
    nout_sum = SHAPE[0] * SHAPE[2]
    nout_arg = SHAPE[0] * SHAPE[1] * SHAPE[2]
    return {
        "to_contig": 2 * N * esize if copy_needed else 0,
        "fma": (3 * N + int(np.prod(CSHAPE))) * esize,
        "sum": (N + nout_sum) * esize,
        "argmax": N * esize + nout_arg * 8,
    }


# ------------------------------------------------------------------ clocks


class ClockSampler:
    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            dev = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or "0"
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={dev}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        try:
            rows = [l.split(",") for l in Path(self.path).read_text().strip().splitlines() if l.strip()]
        except Exception:
            return out
        sm = [float(r[1]) for r in rows if len(r) > 8 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 8 and r[2].strip().replace(".", "").isdigit()]
        if sm:
            out["sm_mhz"] = float(np.median(sm))
            out["sm_max_mhz"] = max(mx) if mx else None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            if len(r) > 8:
                for i, nm in enumerate(names):
                    if "Active" in r[5 + i] and "Not" not in r[5 + i]:
                        reasons.add(nm)
        out["reasons"] = sorted(reasons)
        out["samples"] = len(rows)
        return out


# --------------------------------------------------------- GPU workload


class Workload:
    """Device buffers of one step and the calls that run it."""

    def __init__(self, dev, lib, seed=0, dtypes=None, layouts=None):
        import rstsr_gb300 as rt
        from rstsr_gb300._lib import Layout, dtype_code

        self.dev, self.lib, self.rt = dev, lib, rt
        self.cases = []
        self.Layout = Layout
        for di, (dname, dt) in enumerate(DTYPES):
            if dtypes and dname not in dtypes:
                continue
            code = dtype_code(dt)
            esize = np.dtype(dt).itemsize
            cbuf = host_data(dt, int(np.prod(CSHAPE)), seed + 100 + di)
            c_t = rt.asarray(cbuf.reshape(CSHAPE), dev)
            for li, kind in enumerate(LAYOUTS):
                if layouts and kind not in layouts:
                    continue
                blen, stride, off = layout_of(kind, SHAPE)
                ha = host_data(dt, blen, seed + 10 * di + li)
                hb = host_data(dt, blen, seed + 1000 + 10 * di + li)
                a = rt.from_host_layout(ha, SHAPE, stride, off, dev)
                b = rt.from_host_layout(hb, SHAPE, stride, off, dev)
                pshape, pstride = permuted_view(SHAPE, stride)
                la_perm = Layout.make(pshape, pstride, off)
                out_perm = rt.empty(pshape, code, dev, order="C")
                # fused a*b+c: the output layout of `&a * &b`
                d_t = rt.fma(a, b, c_t)
                lab = d_t.layout()
                lc_b = c_t.broadcast_to(SHAPE).layout()
                sum_out = rt.empty((SHAPE[0], SHAPE[2]), code, dev, order="K", like=a.i((slice(None), 0, slice(None), 0)))
                arg_out = rt.empty(SHAPE[:3], np.uint64, dev, order="K", like=a.i((slice(None), slice(None), slice(None), 0)))
                self.cases.append(dict(
                    dname=dname, kind=kind, code=code, esize=esize, a=a, b=b, c=c_t, d=d_t, la=a.layout(),
                    lb=b.layout(), lab=lab, lcb=lc_b, la_perm=la_perm, out_perm=out_perm,
                    copy=(kind != "perm"), sum_out=sum_out, arg_out=arg_out, ha=ha, hb=hb, hc=cbuf,
                    bytes=op_bytes(esize, kind),
                ))
        self.ax_sum = (C.c_int64 * 2)(1, 3)
        self.ax_arg = (C.c_int64 * 1)(3)

    def total_bytes(self):
        return sum(sum(c["bytes"].values()) for c in self.cases)

    def run_op(self, c, op):
        L, ctx = self.lib, self.dev.ctx
        if op == "to_contig":
            if c["copy"]:
                rc = L.rstsr_cuda_assign_arbitrary(ctx, C.c_void_p(c["out_perm"].ptr), C.byref(c["out_perm"].layout()),
                                                   c["code"], C.c_void_p(c["a"].ptr), C.byref(c["la_perm"]), c["code"], 0)
            else:
                rc = 0
        elif op == "fma":
            rc = L.rstsr_cuda_fma(ctx, c["code"], C.c_void_p(c["d"].ptr), C.byref(c["lab"]), C.c_void_p(c["a"].ptr),
                                  C.byref(c["la"]), C.c_void_p(c["b"].ptr), C.byref(c["lb"]), C.c_void_p(c["c"].ptr),
                                  C.byref(c["lcb"]))
        elif op == "sum":
            rc = L.rstsr_cuda_reduce_axes_into(ctx, 0, c["code"], C.c_void_p(c["a"].ptr), C.byref(c["la"]), self.ax_sum, 2,
                                               C.c_void_p(c["sum_out"].ptr), C.byref(c["sum_out"].layout()))
        else:
            rc = L.rstsr_cuda_argreduce_axes_into(ctx, 1, c["code"], C.c_void_p(c["a"].ptr), C.byref(c["la"]),
                                                  self.ax_arg, 1, C.c_void_p(c["arg_out"].ptr),
                                                  C.byref(c["arg_out"].layout()))
        if rc != 0:
            raise RuntimeError(L.rstsr_cuda_last_error().decode())

    def step(self):
        for c in self.cases:
            for op in ("to_contig", "fma", "sum", "argmax"):
                self.run_op(c, op)


def run_gpu(args):
    import torch

    import rstsr_gb300 as rt

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    lib = rt.lib()
    dev = rt.DeviceCuda(local)
    # one explicit (non-default) stream carries every library launch and the
    # timing events
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    dev.set_stream(stream.cuda_stream)
    wl = Workload(dev, lib, seed=0, dtypes=args.dtypes.split(",") if args.dtypes else None,
                  layouts=args.layouts.split(",") if args.layouts else None)
    torch.cuda.synchronize()

    def barrier():
        replicas.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        wl.step()
    barrier()
    l0 = dev.launch_count()
    # the clock samples (summarised in the JSON line) go to RSTSR_BENCH_OUT, else the temp directory
    out_dir = Path(os.environ.get("RSTSR_BENCH_OUT", tempfile.gettempdir()))
    out_dir.mkdir(parents=True, exist_ok=True)
    clocks = ClockSampler(str(out_dir / f"clocks_r{rank}.csv")) if rank == 0 else None
    if clocks:
        clocks.__enter__()
        time.sleep(0.3)  # let the sampler start before the timed region
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        wl.step()
    ev1.record(stream)
    barrier()
    if clocks:
        clocks.__exit__()
    launches = dev.launch_count() - l0
    step_bytes = wl.total_bytes()
    rate, t_s = replicas.whole_job_rate(step_bytes, ev0.elapsed_time(ev1) / args.steps * 1e-3, "cuda")
    t_ms = t_s * 1e3
    value = rate / 1e9

    # per-operation timing (dominant kernel for the roofline), same stream
    per_op = {}
    for op in ("to_contig", "fma", "sum", "argmax"):
        reps = 3
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0 = dev.launch_count()
        e0.record(stream)
        for _ in range(reps):
            for c in wl.cases:
                wl.run_op(c, op)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        by = sum(c["bytes"][op] for c in wl.cases)
        per_op[op] = dict(ms=round(ms, 4), gbs=round(by / (ms * 1e-3) / 1e9, 1), bytes=by,
                          launches=(dev.launch_count() - n0) // reps)
    # per (dtype, layout, op) GB/s
    per_case = {}
    for c in wl.cases:
        for op in ("to_contig", "fma", "sum", "argmax"):
            if c["bytes"][op] == 0:
                continue
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(3):
                wl.run_op(c, op)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / 3
            per_case[f"{c['dname']}/{c['kind']}/{op}"] = round(c["bytes"][op] / (ms * 1e-3) / 1e9, 0)
    # f64 C-contiguous fma alone: the single dominant kernel
    dom = next((c for c in wl.cases if c["dname"] == "f64" and c["kind"] == "c"), wl.cases[0])
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record(stream)
    for _ in range(reps):
        wl.run_op(dom, "fma")
    e1.record(stream)
    torch.cuda.synchronize()
    fma_ms = e0.elapsed_time(e1) / reps
    fma_bytes = dom["bytes"]["fma"]

    e2e = run_e2e(wl, dev, stream, args, world) if not args.no_e2e else None
    result = None
    if rank == 0:
        peaks = {}
        try:
            peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        except Exception:
            pass
        peak = peaks.get("hbm_gbs", 6800.0)
        achieved = fma_bytes / (fma_ms * 1e-3) / 1e9
        traffic = None
        tpath = ROOT / "profiles" / "traffic.json"
        if tpath.exists():
            try:
                traffic = json.loads(tpath.read_text()).get("fma_f64_c")
            except Exception:
                traffic = None
        details = {"per_op": per_op, "per_case": per_case}
        result = {
            "metric": METRIC,
            "value": round(value, 1),
            "unit": "GB/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(t_ms, 4),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64,f32,i32",
            "data": "synthetic (seeded uniform; i32 uniform in [-1000,1000])",
            "gpu_launches": int(launches),
            "config": {
                "workload": WORKLOAD,
                "l2": "inputs larger than L2 (>=128 MiB per tensor), no flush",
                "parallelism": f"replicas x{world}",
                "step_bytes": step_bytes,
            },
            "roofline": {
                "kernel": "fma (a*b+c, f64, C-contiguous, broadcast c)",
                "bound": "hbm",
                "achieved": round(achieved, 1),
                "peak": peak,
                "unit": "GB/s",
                "frac": round(achieved / peak, 3),
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "fallback",
                "traffic": traffic,
                "algorithmic_bytes_per_launch": fma_bytes,
                "avg_launch_ms": round(fma_ms, 4),
            },
            "e2e": e2e,
            "clocks": clocks.summary() if clocks else None,
            # fraction of the measured HBM bandwidth per operation over all cases
            "per_op_frac_hbm": {op: round(v["gbs"] / peak, 3) for op, v in per_op.items()},
        }
        if not args.no_cpu:
            result["cpu_baseline"], result["parity"] = cpu_baseline(args, wl)
        if not args.no_gemm:
            gemm = run_gemm_section(dev, stream)
            gemm.update(run_batched_section(dev, stream))
            details["gemm"] = gemm
            details["small_f64"] = run_small_section(dev, stream)
            details["tri_index"] = run_tri_index_section(dev, stream)
            details["contraction"] = run_contraction_section(dev, stream)
            details["contraction"].update(run_blas3_section(dev, stream))
            result["details_file"] = "bench_details.json (RSTSR_BENCH_OUT, else the temp directory)"
            # the GEMM half of the metric, compact and last on the line
            result["gemm"] = gemm_summary(gemm, details["small_f64"])
        (out_dir / "bench_details.json").write_text(json.dumps(details, indent=1))
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    return result


def gemm_summary(g, small):
    """The headline GEMM numbers (full entries in the details file)."""
    c3 = g["c3_ozaki_f64"]
    out = {}
    for name in ("c4_split_f32_8192", "c4_split_f32_tall"):
        e = g[name]
        out[name] = {"tflops": e["tflops"], "rel_err": float(f"{e['rel_err_vs_fp64']:.3g}"), "tuned": True,
                     "sgemm_tflops": e["cublas_sgemm_tflops"],
                     "bf16x9_tflops": e.get("cublas_emulated_bf16x9", {}).get("tflops")}
    gr, bc, ch = g["c5_grouped_f64_512"], g["c5_broadcast_batch_f64"], g["c5_graph_chain_f64"]
    out["c5"] = {"grouped_tflops": gr["tflops"], "grouped_err": float(f"{gr['rel_err_frobenius']:.3g}"),
                 "grouped_launches": gr["launches_per_call"], "tuned": gr.get("tuned", False),
                 "bcast_tflops": bc["tflops"], "bcast_err": float(f"{bc['rel_err_frobenius']:.3g}"),
                 "graph_us": ch["graph_us_per_iter"], "eager_us": ch["eager_us_per_iter"]}
    out["c1_small_f64"] = {"exact_add": small["add_bit_exact"], "exact_argmax": small["argmax_exact"],
                           "matmul_err": float(f"{small['matmul_rel_err']:.3g}"),
                           "eager_us": [small["add_us"], small["sum_axes_us"], small["argmax_axes_us"], small["matmul_us"]],
                           "graph_4ops_us": small["graph_4ops_us"]}
    out["c3_ozaki_f64"] = {
        "tflops": c3["tflops"], "ms": c3["ms"], "slices": c3["slices"],
        "rel_err": float(f"{c3['rel_err_frobenius']:.3g}"),
        "dgemm_tflops": c3["native_fp64_cublas_tflops"], "dsyrk_tflops": c3.get("native_dsyrk_tflops"),
        "speedup_vs_dgemm": c3["speedup_vs_native_fp64"], "speedup_vs_dsyrk": c3.get("speedup_vs_native_dsyrk"),
        "tensor_frac": c3["roofline"]["frac"]}
    return out


def _time_events(stream, fn, reps):
    import torch

    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps * 1e-3


class _CublasEmulated:
    """cuBLAS GEMM with an emulated compute type, a comparator only: FP64
    through fixed-point emulation (CUBLAS_COMPUTE_64F_EMULATED_FIXEDPOINT) and
    FP32 through three bf16 terms (CUBLAS_COMPUTE_32F_EMULATED_16BFX9), with the
    emulation strategy set to always emulate. Column-major, as cuBLAS is."""

    F64_FIXEDPOINT, F32_BF16X9 = 79, 78

    def __init__(self, stream):
        lib = _cublas_lib()
        self.lib = lib
        self.h = C.c_void_p()
        if lib.cublasCreate_v2(C.byref(self.h)) != 0:
            raise RuntimeError("cublasCreate failed")
        lib.cublasSetStream_v2(self.h, C.c_void_p(stream.cuda_stream))
        if lib.cublasSetEmulationStrategy(self.h, 2) != 0:  # CUBLAS_EMULATION_STRATEGY_EAGER
            raise RuntimeError("cublasSetEmulationStrategy failed")
        lib.cublasGemmEx.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                     C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                     C.c_int, C.c_int, C.c_int]

    def gemm(self, ta, tb, m, n, k, a, lda, b, ldb, c, ldc, f64, compute):
        one = C.c_double(1.0) if f64 else C.c_float(1.0)
        zero = C.c_double(0.0) if f64 else C.c_float(0.0)
        dt = 1 if f64 else 0  # CUDA_R_64F / CUDA_R_32F
        st = self.lib.cublasGemmEx(self.h, ta, tb, m, n, k, C.byref(one), C.c_void_p(a), dt, lda, C.c_void_p(b), dt,
                                   ldb, C.byref(zero), C.c_void_p(c), dt, ldc, compute, -1)
        if st != 0:
            raise RuntimeError(f"cublasGemmEx returned {st}")

    def close(self):
        self.lib.cublasDestroy_v2(self.h)


def _cublas_lib():
    for name in ("libcublas.so.13", "/usr/local/cuda/lib64/libcublas.so.13"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    raise RuntimeError("libcublas.so.13 not found")


def _cublas_dsyrk(stream, x, n, k, ref):
    """cuBLAS DSYRK (native FP64) of C = X X^T, X the column-major [n, k] view
    of the row-major [k, n] tensor `x`, lower triangle; returns (seconds,
    relative Frobenius error of that triangle against `ref`)."""
    import torch

    lib = _cublas_lib()
    h = C.c_void_p()
    if lib.cublasCreate_v2(C.byref(h)) != 0:
        raise RuntimeError("cublasCreate failed")
    try:
        lib.cublasSetStream_v2(h, C.c_void_p(stream.cuda_stream))
        lib.cublasDsyrk_v2.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                       C.c_void_p, C.c_void_p, C.c_int]
        c = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        one, zero = C.c_double(1.0), C.c_double(0.0)

        def run():
            st = lib.cublasDsyrk_v2(h, 0, 0, n, k, C.byref(one), C.c_void_p(x.data_ptr()), n, C.byref(zero),
                                    C.c_void_p(c.data_ptr()), n)
            if st != 0:
                raise RuntimeError(f"cublasDsyrk returned {st}")

        sec = _time_events(stream, run, 1)
        # the column-major lower triangle is the upper triangle of the row-major view
        tri = torch.triu(c)
        rtri = torch.triu(ref)
        err = (torch.linalg.norm(tri - rtri) / torch.linalg.norm(rtri)).item()
        del c, tri, rtri
        return sec, err
    finally:
        lib.cublasDestroy_v2(h)


def run_gemm_section(dev, stream):
    """The GEMM half of the metric: the f64 electronic-structure contraction
    C = Bm^T Bm (Bm = B[P=1000, i=50, a=300] reshaped to 1000 x 15000, entries
    N(0,1) exp(-0.01 P), seed 0) through the Ozaki split against native FP64
    (cuBLAS DGEMM on the same GPU, also the FP64 oracle for the error), and the
    f32 three-term bf16 split on 8192^3 and 65536x256x256 (entries
    U(-1,1) 2^U(-8,8)) against cuBLAS SGEMM, errors against FP64."""
    import torch

    import rstsr_gb300 as rt

    out = {}
    rng = np.random.default_rng(0)
    P, Q = 1000, 50 * 300
    bm = rng.standard_normal((P, Q)) * np.exp(-0.01 * np.arange(P))[:, None]
    t = rt.asarray(bm, dev)
    c = rt.empty((Q, Q), np.float64, dev)
    run = lambda: rt.matmul_into(c, t.t(), t, 1.0, 0.0)
    sec = _time_events(stream, run, 3)
    slices = int(rt.lib().rstsr_cuda_last_ozaki_slices())
    flops = 2.0 * Q * Q * P
    tb = torch.from_numpy(bm).cuda()
    ref = tb.T @ tb
    sec_ref = _time_events(stream, lambda: tb.T @ tb, 1)
    got = torch.as_tensor(c.to_numpy()).cuda()
    err = (torch.linalg.norm(got - ref) / torch.linalg.norm(ref)).item()
    # tensor work of the split kernel: L(L+1)/2 bf16 slice products on every
    # computed 128x64 tile (lower triangle of the symmetric product), K padded
    # to 16; against the measured cuBLAS bf16 peak (the whole call is timed, so
    # the statistics and split kernels count against it)
    tiles_m, tiles_n = -(-Q // 128), -(-Q // 64)
    ntiles = sum(tiles_m - j // 2 for j in range(min(2 * tiles_m, tiles_n)))
    bf16_flops = 2.0 * ntiles * 128 * 64 * (-(-P // 16) * 16) * slices * (slices + 1) // 2
    try:
        peak = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["bf16_tflops"])
        peak_src = "measured (MEASURED_PEAKS.json bf16_tflops)"
    except Exception:
        peak, peak_src = 1900.0, "fallback"
    out["c3_ozaki_f64"] = {
        "shape": "Bm^T Bm, m=n=15000, k=1000 (SYRK path)", "tflops": round(flops / sec / 1e12, 2),
        "ms": round(sec * 1e3, 3), "slices": slices, "rel_err_frobenius": err,
        "native_fp64_cublas_tflops": round(flops / sec_ref / 1e12, 3), "native_ms": round(sec_ref * 1e3, 2),
        "speedup_vs_native_fp64": round(sec_ref / sec, 1), "flop_count": "2mnk (full product)",
        "roofline": {"bound": "tensor", "achieved": round(bf16_flops / sec / 1e12, 1), "peak": peak,
                     "unit": "TFLOP/s", "frac": round(bf16_flops / sec / 1e12 / peak, 3),
                     "peak_source": peak_src, "work": "bf16 slice products of the computed tiles"},
    }
    # native comparator on the reference's own path (SYRK: only one triangle
    # is computed, as the reference's B^T B does): cuBLAS DSYRK, C = X X^T with
    # X the column-major [15000, 1000] view of Bm, lower triangle
    try:
        sec_syrk, err_syrk = _cublas_dsyrk(stream, tb, Q, P, ref)
        out["c3_ozaki_f64"].update({
            "native_dsyrk_tflops": round(flops / sec_syrk / 1e12, 3), "native_dsyrk_ms": round(sec_syrk * 1e3, 2),
            "native_dsyrk_rel_err_triangle": err_syrk, "speedup_vs_native_dsyrk": round(sec_syrk / sec, 1)})
    except Exception as exc:
        out["c3_ozaki_f64"]["native_dsyrk"] = {"unavailable": str(exc)[:200]}
    # comparator: cuBLAS's own fixed-point FP64 emulation, C = X X^T with X the
    # column-major [15000, 1000] view of Bm
    try:
        cb = _CublasEmulated(stream)
        ce = torch.empty((Q, Q), dtype=torch.float64, device="cuda")
        fn = lambda: cb.gemm(0, 1, Q, Q, P, tb.data_ptr(), Q, tb.data_ptr(), Q, ce.data_ptr(), Q, True,
                             cb.F64_FIXEDPOINT)
        sec_e = _time_events(stream, fn, 1)
        out["c3_ozaki_f64"]["cublas_emulated_fp64_fixedpoint"] = {
            "tflops": round(flops / sec_e / 1e12, 2), "ms": round(sec_e * 1e3, 3),
            "rel_err_frobenius": (torch.linalg.norm(ce - ref) / torch.linalg.norm(ref)).item()}
        del ce
        cb.close()
    except Exception as exc:  # the comparator is optional
        out["c3_ozaki_f64"]["cublas_emulated_fp64_fixedpoint"] = {"unavailable": str(exc)[:200]}
    # CPU baseline: host BLAS dsyrk (the DeviceOpenBLAS call) on a bounded sample
    try:
        from scipy.linalg import blas as sblas

        qs = 3000
        xs = np.ascontiguousarray(bm[:, :qs])
        sblas.dsyrk(1.0, xs, trans=1)
        t0 = time.perf_counter()
        sblas.dsyrk(1.0, xs, trans=1)
        tc = time.perf_counter() - t0
        out["c3_ozaki_f64"]["cpu_baseline"] = {
            "value": round(2.0 * qs * qs * P / tc / 1e12, 4), "unit": "TFLOP/s", "cores": os.cpu_count(),
            "kind": "host BLAS dsyrk (scipy)", "sample": f"Bm[:, :{qs}]^T Bm[:, :{qs}], 2mnk flops"}
    except Exception as exc:
        out["c3_ozaki_f64"]["cpu_baseline"] = {"unavailable": str(exc)[:200]}
    del c, ref, got, tb
    torch.cuda.empty_cache()
    for name, (m, n, k) in (("c4_split_f32_8192", (8192, 8192, 8192)), ("c4_split_f32_tall", (65536, 256, 256))):
        a = (rng.uniform(-1, 1, (m, k)) * 2.0 ** rng.uniform(-8, 8, (m, k))).astype(np.float32)
        b = (rng.uniform(-1, 1, (k, n)) * 2.0 ** rng.uniform(-8, 8, (k, n))).astype(np.float32)
        ta, tb2 = rt.asarray(a, dev), rt.asarray(b, dev)
        c = rt.empty((m, n), np.float32, dev)
        # tile configuration from the project's autotuner for this shape class
        code = rt.autotune_gemm(dev, np.float32, m, n, k)
        sec = _time_events(stream, lambda: rt.matmul_into(c, ta, tb2), 3)
        fa, fb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
        ref = fa.double() @ fb.double()
        torch.backends.cuda.matmul.allow_tf32 = False
        sec_s = _time_events(stream, lambda: fa @ fb, 3)
        sref = (fa @ fb).double()
        got = torch.as_tensor(c.to_numpy()).cuda().double()
        nr = torch.linalg.norm(ref)
        out[name] = {
            "shape": f"{m}x{n}x{k}", "tflops": round(2.0 * m * n * k / sec / 1e12, 2), "ms": round(sec * 1e3, 3),
            "tuned_config": {"k_tile": code & 255, "group": code >> 8},
            "rel_err_vs_fp64": (torch.linalg.norm(got - ref) / nr).item(),
            "cublas_sgemm_tflops": round(2.0 * m * n * k / sec_s / 1e12, 2),
            "cublas_sgemm_rel_err_vs_fp64": (torch.linalg.norm(sref - ref) / nr).item(),
        }
        try:  # comparator: cuBLAS BF16x9 emulation of FP32 (row-major C = A B as col-major C^T = B^T A^T)
            cb = _CublasEmulated(stream)
            ce = torch.empty((m, n), dtype=torch.float32, device="cuda")
            fn = lambda: cb.gemm(0, 0, n, m, k, fb.data_ptr(), n, fa.data_ptr(), k, ce.data_ptr(), n, False,
                                 cb.F32_BF16X9)
            sec_e = _time_events(stream, fn, 3)
            out[name]["cublas_emulated_bf16x9"] = {
                "tflops": round(2.0 * m * n * k / sec_e / 1e12, 2), "ms": round(sec_e * 1e3, 3),
                "rel_err_vs_fp64": (torch.linalg.norm(ce.double() - ref) / nr).item()}
            del ce
            cb.close()
        except Exception as exc:
            out[name]["cublas_emulated_bf16x9"] = {"unavailable": str(exc)[:200]}
        del a, b, ta, tb2, c, fa, fb, ref, sref, got
        torch.cuda.empty_cache()
    return out


def run_rates(args):
    """Dense tensor-core rates that decide the slice type of the split GEMMs
    on this GPU: INT8 (torch._int_mm, int32 accumulation), BF16 and FP16
    (torch.matmul, fp32 accumulation) and native FP64 (torch.matmul, cuBLAS
    DGEMM), all n^3 with n = --rate-n, CUDA events, best of the timed calls."""
    import torch

    n = args.rate_n
    stream = torch.cuda.current_stream()
    res = {"n": n}
    g = torch.Generator(device="cuda").manual_seed(0)

    def best(fn, reps):
        fn()
        torch.cuda.synchronize()
        t = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            t.append(e0.elapsed_time(e1) * 1e-3)
        return min(t)

    a8 = torch.randint(-128, 128, (n, n), dtype=torch.int8, device="cuda", generator=g)
    b8 = torch.randint(-128, 128, (n, n), dtype=torch.int8, device="cuda", generator=g)
    try:
        res["int8_tops"] = round(2.0 * n ** 3 / best(lambda: torch._int_mm(a8, b8), 10) / 1e12, 1)
    except Exception as exc:
        res["int8_tops"] = f"unavailable: {str(exc)[:120]}"
    del a8, b8
    for name, dt in (("bf16_tflops", torch.bfloat16), ("fp16_tflops", torch.float16)):
        x = torch.rand((n, n), dtype=dt, device="cuda", generator=g)
        y = torch.rand((n, n), dtype=dt, device="cuda", generator=g)
        res[name] = round(2.0 * n ** 3 / best(lambda: x @ y, 10) / 1e12, 1)
        del x, y
    x = torch.rand((n, n), dtype=torch.float64, device="cuda", generator=g)
    y = torch.rand((n, n), dtype=torch.float64, device="cuda", generator=g)
    res["fp64_tflops"] = round(2.0 * n ** 3 / best(lambda: x @ y, 2) / 1e12, 3)
    res["torch"] = torch.__version__
    res["gpu"] = torch.cuda.get_device_name(0)
    return {"section": "tensor_rates", "results": res}


def run_c3_only(args):
    """Only the Ozaki contraction C = Bm^T Bm with Bm [1000, cols] (cols =
    15000 is the full workload; smaller for profiling), timed over --steps
    calls after --warmup; one JSON line."""
    import torch

    import rstsr_gb300 as rt

    dev = rt.DeviceCuda(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    dev.set_stream(stream.cuda_stream)
    rng = np.random.default_rng(0)
    P, Q = 1000, args.c3_cols
    bm = rng.standard_normal((P, Q)) * np.exp(-0.01 * np.arange(P))[:, None]
    t = rt.asarray(bm, dev)
    c = rt.empty((Q, Q), np.float64, dev)
    for _ in range(max(args.warmup - 1, 0)):
        rt.matmul_into(c, t.t(), t, 1.0, 0.0)
    sec = _time_events(stream, lambda: rt.matmul_into(c, t.t(), t, 1.0, 0.0), max(args.steps, 1))
    flops = 2.0 * Q * Q * P
    return {"metric": "f64 Ozaki-split GEMM TFLOP/s", "value": round(flops / sec / 1e12, 2), "unit": "TFLOP/s",
            "ms_per_step": round(sec * 1e3, 3), "steps": args.steps, "warmup": args.warmup,
            "slices": int(rt.lib().rstsr_cuda_last_ozaki_slices()),
            "config": {"workload": f"Bm^T Bm, Bm [1000, {Q}] (SYRK path)"}}


def run_batched_section(dev, stream):
    """Batched / grouped matmul and the graph-captured op chain:
    (i) 512 f64 GEMMs with m, n, k uniform in [16, 512] (seed 0) as one grouped
    launch; (ii) the broadcast batch [64,1,256,256] % [1,32,256,256] f64
    (2048 products, matmul rule 7); (iii) matmul [256,256] % [256,256] ->
    broadcast bias add [256] -> sum_axes(1), f64, captured once as a CUDA graph
    and replayed 1000 times, against the same chain issued eagerly."""
    import ctypes as C

    import torch

    import rstsr_gb300 as rt
    from rstsr_gb300._lib import GemmProblem, call

    out = {}
    rng = np.random.default_rng(0)
    # (i) uneven grouped
    dims = rng.integers(16, 513, (512, 3))
    probs, keep, flops = [], [], 0.0
    for m, n, k in dims:
        m, n, k = int(m), int(n), int(k)
        a = rng.uniform(-1, 1, (m, k))
        b = rng.uniform(-1, 1, (k, n))
        ta, tb = rt.asarray(a, dev), rt.asarray(b, dev)
        tc = rt.empty((m, n), np.float64, dev)
        keep.append((a, b, ta, tb, tc))
        probs.append(GemmProblem(m, n, k, k, n, n, ta.ptr, tb.ptr, tc.ptr, 1.0, 0.0))
        flops += 2.0 * m * n * k
    arr = (GemmProblem * len(probs))(*probs)
    run = lambda: call("rstsr_cuda_gemm_grouped", dev.ctx, 0, arr, len(probs), None)
    run()
    torch.cuda.synchronize()
    # tile configuration from the project's autotuner, for the shape class of
    # the call (its largest m, n, k) at the slice count the call chose
    sl = int(rt.lib().rstsr_cuda_last_ozaki_slices())
    mx = [int(v) for v in dims.max(axis=0)]
    tuned = rt.autotune_gemm(dev, np.float64, mx[0], mx[1], mx[2], slices=sl)
    l0 = dev.launch_count()
    run()
    torch.cuda.synchronize()
    launches = dev.launch_count() - l0
    sec = _time_events(stream, run, 5)
    num = den = 0.0
    for a, b, _, _, tc in keep:
        r = a @ b
        num += float(np.sum((tc.to_numpy() - r) ** 2))
        den += float(np.sum(r * r))
    out["c5_grouped_f64_512"] = {"tflops": round(flops / sec / 1e12, 2), "ms": round(sec * 1e3, 3),
                                 "sum_2mnk": flops, "rel_err_frobenius": (num / den) ** 0.5,
                                 "launches_per_call": int(launches), "slices": sl, "tuned": True,
                                 "tuned_config": {"shape_class": mx, "k_tile": tuned & 0xFF, "group": tuned >> 8}}
    del keep, probs, arr
    # (ii) broadcast batch
    a = rng.uniform(-1, 1, (64, 1, 256, 256))
    b = rng.uniform(-1, 1, (1, 32, 256, 256))
    ta, tb = rt.asarray(a, dev), rt.asarray(b, dev)
    tc = rt.empty((64, 32, 256, 256), np.float64, dev)
    run = lambda: rt.matmul_into(tc, ta, tb)
    run()
    torch.cuda.synchronize()
    sl = int(rt.lib().rstsr_cuda_last_ozaki_slices())
    tuned = rt.autotune_gemm(dev, np.float64, 256, 256, 256, slices=sl)
    l0 = dev.launch_count()
    run()
    torch.cuda.synchronize()
    launches = dev.launch_count() - l0
    sec = _time_events(stream, run, 3)
    ga, gb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    ref = torch.matmul(ga, gb)
    sec_ref = _time_events(stream, lambda: torch.matmul(ga, gb), 1)
    got = torch.as_tensor(tc.to_numpy()).cuda()
    flops = 2.0 * 2048 * 256 ** 3
    out["c5_broadcast_batch_f64"] = {
        "shape": "[64,1,256,256] % [1,32,256,256]", "tflops": round(flops / sec / 1e12, 2), "ms": round(sec * 1e3, 3),
        "rel_err_frobenius": (torch.linalg.norm(got - ref) / torch.linalg.norm(ref)).item(),
        "native_fp64_cublas_tflops": round(flops / sec_ref / 1e12, 3), "launches_per_call": int(launches),
        "slices": sl, "tuned": True, "tuned_config": {"k_tile": tuned & 0xFF, "group": tuned >> 8}}
    del ta, tb, tc, ga, gb, ref, got
    torch.cuda.empty_cache()
    # (iii) graph-captured chain
    a = rng.uniform(-1, 1, (256, 256))
    b = rng.uniform(-1, 1, (256, 256))
    bias = rng.uniform(-1, 1, (256,))
    ta, tb, tbias = rt.asarray(a, dev), rt.asarray(b, dev), rt.asarray(bias, dev)
    c = rt.empty((256, 256), np.float64, dev)
    o = rt.empty((256,), np.float64, dev)

    def chain():
        rt.matmul_into(c, ta, tb, 1.0, 0.0, slices=7)
        rt.binary_inplace("add", c, tbias)
        rt.reduce_axes_into("sum", c, [1], o)

    chain()
    eager_us = _time_events(stream, chain, 100) * 1e6
    with rt.Graph(dev) as g:
        chain()
    g.launch()
    graph_us = _time_events(stream, g.launch, 1000) * 1e6
    want = (a @ b + bias).sum(axis=1)
    err = float(np.linalg.norm(o.to_numpy() - want) / np.linalg.norm(want))
    out["c5_graph_chain_f64"] = {"chain": "[256,256]%[256,256] + bias[256] -> sum_axes(1)", "replays": 1000,
                                 "graph_us_per_iter": round(graph_us, 2), "eager_us_per_iter": round(eager_us, 2),
                                 "rel_err": err}
    return out


def capture_small_ops(dev, tA, tb, tB):
    """Capture C = A + b, sum_axes(C, 1), argmax_axes(C, 1) and A % B into
    caller-owned outputs as one CUDA graph. Returns the graph and the outputs
    (C, sums, argmax indices, product)."""
    import rstsr_gb300 as rt
    from rstsr_gb300 import _lib
    from rstsr_gb300.tensor import broadcast_layouts

    la, lb = broadcast_layouts(tA, tb, dev.default_order)
    cbuf = rt.empty((tA.shape[0], tA.shape[1]), np.float64, dev)
    s_out = rt.empty((tA.shape[0],), np.float64, dev)
    g_out = rt.empty((tA.shape[0],), np.uint64, dev)
    m_out = rt.empty((tA.shape[0], tB.shape[1]), np.float64, dev)
    ax = (C.c_int64 * 1)(1)

    def ops():
        _lib.call("rstsr_cuda_binary", dev.ctx, _lib.OP["add"], cbuf.dtype_code, C.c_void_p(cbuf.ptr),
                  C.byref(cbuf.layout()), C.c_void_p(tA.ptr), C.byref(la), C.c_void_p(tb.ptr), C.byref(lb))
        rt.reduce_axes_into("sum", cbuf, [1], s_out)
        _lib.call("rstsr_cuda_argreduce_axes_into", dev.ctx, 1, cbuf.dtype_code, C.c_void_p(cbuf.ptr),
                  C.byref(cbuf.layout()), ax, 1, C.c_void_p(g_out.ptr), C.byref(g_out.layout()))
        rt.matmul_into(m_out, tA, tB)

    ops()  # first call outside the capture: workspaces are sized here
    with rt.Graph(dev) as g:
        ops()
    return g, (cbuf, s_out, g_out, m_out)


def run_small_section(dev, stream):
    """The small f64 row-major case: A [64,128] and b [128] uniform(-1,1),
    B [128,96]; C = A + b, sum_axes(C, 1), argmax_axes(C, 1), A % B. Device
    latency per operation (events, inputs resident) and the errors."""
    import rstsr_gb300 as rt

    rng = np.random.default_rng(0)
    A = rng.uniform(-1, 1, (64, 128))
    b = rng.uniform(-1, 1, (128,))
    B = rng.uniform(-1, 1, (128, 96))
    tA, tb, tB = rt.asarray(A, dev), rt.asarray(b, dev), rt.asarray(B, dev)
    Cd = tA + tb
    res = {}
    res["add_us"] = round(_time_events(stream, lambda: tA + tb, 200) * 1e6, 2)
    res["sum_axes_us"] = round(_time_events(stream, lambda: Cd.sum_axes(1), 200) * 1e6, 2)
    res["argmax_axes_us"] = round(_time_events(stream, lambda: Cd.argmax_axes(1), 200) * 1e6, 2)
    res["matmul_us"] = round(_time_events(stream, lambda: rt.matmul(tA, tB), 50) * 1e6, 2)
    C = A + b
    res["add_bit_exact"] = bool(np.array_equal(Cd.to_numpy(), C))
    s = Cd.sum_axes(1).to_numpy()
    res["sum_rel_err"] = float(np.max(np.abs(s - C.sum(axis=1))) / np.max(np.abs(C.sum(axis=1))))
    res["argmax_exact"] = bool(np.array_equal(Cd.argmax_axes(1).to_numpy(), np.argmax(C, axis=1)))
    m = rt.matmul(tA, tB).to_numpy()
    res["matmul_rel_err"] = float(np.linalg.norm(m - A @ B) / np.linalg.norm(A @ B))
    # the same four operations into caller-owned outputs, captured once as a
    # CUDA graph and replayed: the device time of the library's launches
    # without the Python / ctypes call overhead of the eager figures above
    g, outs = capture_small_ops(dev, tA, tb, tB)
    g.launch()
    res["graph_4ops_us"] = round(_time_events(stream, g.launch, 200) * 1e6, 2)
    cbuf, _, g_out, _ = outs
    res["graph_bit_exact"] = bool(np.array_equal(cbuf.to_numpy(), C)) and bool(
        np.array_equal(g_out.to_numpy(), np.argmax(C, axis=1)))
    return res


def run_tri_index_section(dev, stream, n=2048, batch=32, rows=16384, cols=8192):
    """Packed-triangle and index-selection kernels on resident f64 data:
    pack_tri 'L' of [batch, n, n] (read the triangle, write the packed
    vector: 2 * batch * n(n+1)/2 * 8 bytes), unpack_tri 'L' Sy of the packed
    [batch, n(n+1)/2] (read it once, write both triangles: batch *
    (n(n+1)/2 + n^2) * 8 bytes), and index_select of half the rows (axis 0)
    and half the columns (axis 1) of a [rows, cols] matrix, random indices
    with repeats (read + write of the selected elements). Device time by CUDA
    events, inputs larger than L2; torch's gather on the same data beside it."""
    import torch

    import rstsr_gb300 as rt

    peak = 6800.0
    try:
        peak = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("hbm_gbs", peak)
    except Exception:
        pass
    out = {}
    rng = np.random.default_rng(0)
    ntp = n * (n + 1) // 2

    def entry(name, sec, nbytes, launches, torch_sec=None, **kw):
        gbs = nbytes / sec / 1e9
        e = {"gbs": round(gbs, 1), "ms": round(sec * 1e3, 4), "bytes": int(nbytes), "frac_hbm": round(gbs / peak, 3),
             "launches_per_call": int(launches)}
        if torch_sec:
            e["torch_gbs"] = round(nbytes / torch_sec / 1e9, 1)
        e.update(kw)
        out[name] = e

    m = rng.standard_normal((batch, n, n))
    tm = rt.asarray(m, dev)
    del m
    l0 = dev.launch_count()
    packed = rt.pack_tri(tm, "L")
    torch.cuda.synchronize()
    launches = dev.launch_count() - l0
    sec = _time_events(stream, lambda: rt.pack_tri(tm, "L"), 5)
    gm = torch.empty((batch, n, n), dtype=torch.float64, device="cuda")
    il = torch.tril_indices(n, n, device="cuda")
    sec_t = _time_events(stream, lambda: gm[:, il[0], il[1]], 3)
    entry("pack_tril_f64", sec, 2 * batch * ntp * 8, launches, sec_t, shape=[batch, n, n])
    del gm
    l0 = dev.launch_count()
    rt.unpack_tri(packed, "L", "Sy")
    torch.cuda.synchronize()
    launches = dev.launch_count() - l0
    sec = _time_events(stream, lambda: rt.unpack_tri(packed, "L", "Sy"), 5)
    entry("unpack_tril_sy_f64", sec, batch * (ntp + n * n) * 8, launches, shape=[batch, ntp])
    del tm, packed, il
    torch.cuda.empty_cache()

    a = rng.standard_normal((rows, cols))
    ta = rt.asarray(a, dev)
    ga = torch.from_numpy(a).cuda()
    del a
    ridx = rng.integers(0, rows, rows // 2)
    l0 = dev.launch_count()
    rt.index_select(ta, 0, ridx)
    torch.cuda.synchronize()
    launches = dev.launch_count() - l0
    sec = _time_events(stream, lambda: rt.index_select(ta, 0, ridx), 5)
    gidx = torch.from_numpy(ridx).cuda()
    sec_t = _time_events(stream, lambda: torch.index_select(ga, 0, gidx), 5)
    entry("index_select_rows_f64", sec, 2 * (rows // 2) * cols * 8, launches, sec_t, shape=[rows, cols],
          indices=rows // 2)
    cidx = rng.integers(0, cols, cols // 2)
    sec = _time_events(stream, lambda: rt.index_select(ta, 1, cidx), 5)
    gidx = torch.from_numpy(cidx).cuda()
    sec_t = _time_events(stream, lambda: torch.index_select(ga, 1, gidx), 5)
    entry("index_select_cols_f64", sec, 2 * rows * (cols // 2) * 8, launches, sec_t, shape=[rows, cols],
          indices=cols // 2)
    del ta, ga
    torch.cuda.empty_cache()
    return out


def run_contraction_section(dev, stream, P=1000, nao=350, nocc=50, nvir=300, vec_rows=8192, vec_cols=8192):
    """The 3-index AO -> MO transform B[P, i, a] = sum_mn B[P, m, n] Co[m, i] Cv[n, a]
    (f64, synthetic seeded inputs; P = 1000, nao = 350, nocc = 50, nvir = 300:
    the B[1000, 50, 300] that the Ozaki SYRK then contracts), through einsum:
    two batched split GEMMs (2*P*nao*nao*nocc + 2*P*nocc*nao*nvir flop), against
    torch.einsum in FP64 (cuBLAS DGEMM) on the same data and the relative
    Frobenius error against that FP64 result; plus vecdot of two
    [vec_rows, vec_cols] f64 arrays along the last axis (HBM-bound: 2 reads)."""
    import torch

    import rstsr_gb300 as rt

    out = {}
    rng = np.random.default_rng(0)
    B = rng.standard_normal((P, nao, nao)) * np.exp(-0.01 * np.arange(P))[:, None, None]
    Co = rng.standard_normal((nao, nocc))
    Cv = rng.standard_normal((nao, nvir))
    tB, tCo, tCv = rt.asarray(B, dev), rt.asarray(Co, dev), rt.asarray(Cv, dev)
    gB, gCo, gCv = torch.from_numpy(B).cuda(), torch.from_numpy(Co).cuda(), torch.from_numpy(Cv).cuda()
    del B
    sub = "Pmn,mi,na->Pia"
    l0 = dev.launch_count()
    res = rt.einsum(sub, tB, tCo, tCv)
    torch.cuda.synchronize()
    launches = dev.launch_count() - l0
    sec = _time_events(stream, lambda: rt.einsum(sub, tB, tCo, tCv), 5)
    ref = torch.einsum("Pmn,mi->Pin", gB, gCo)
    ref = torch.einsum("Pin,na->Pia", ref, gCv)
    sec_t = _time_events(stream, lambda: torch.einsum("Pin,na->Pia", torch.einsum("Pmn,mi->Pin", gB, gCo), gCv), 2)
    got = torch.as_tensor(res.to_numpy()).cuda()
    err = (torch.linalg.norm(got - ref) / torch.linalg.norm(ref)).item()
    flops = 2.0 * P * nao * nao * nocc + 2.0 * P * nocc * nao * nvir
    out["einsum_3index_f64"] = {
        "subscripts": sub, "shapes": [[P, nao, nao], [nao, nocc], [nao, nvir]],
        "tflops": round(flops / sec / 1e12, 2), "ms": round(sec * 1e3, 3), "flop": flops,
        "rel_err_frobenius_vs_fp64": err, "launches_per_call": int(launches),
        "torch_fp64_tflops": round(flops / sec_t / 1e12, 3), "torch_fp64_ms": round(sec_t * 1e3, 3)}
    # host sample: numpy einsum (BLAS) on P = 32 of the 1000 (scaled by P)
    import time as _t
    Bs = rng.standard_normal((32, nao, nao))
    t0 = _t.perf_counter()
    np.einsum(sub, Bs, Co, Cv, optimize=True)
    host = _t.perf_counter() - t0
    out["einsum_3index_f64"]["cpu_numpy_sample"] = {"P": 32, "s": round(host, 4),
                                                   "tflops": round(flops * 32 / P / host / 1e12, 4)}
    del tB, gB, ref, got, res
    torch.cuda.empty_cache()
    a = rng.standard_normal((vec_rows, vec_cols))
    b = rng.standard_normal((vec_rows, vec_cols))
    ta, tb = rt.asarray(a, dev), rt.asarray(b, dev)
    l0 = dev.launch_count()
    v = rt.vecdot(ta, tb)
    torch.cuda.synchronize()
    launches = dev.launch_count() - l0
    sec = _time_events(stream, lambda: rt.vecdot(ta, tb), 5)
    want = np.einsum("ij,ij->i", a, b)
    nbytes = 2 * vec_rows * vec_cols * 8 + vec_rows * 8
    out["vecdot_f64"] = {"shape": [vec_rows, vec_cols], "gbs": round(nbytes / sec / 1e9, 1), "ms": round(sec * 1e3, 4),
                         "launches_per_call": int(launches),
                         "max_rel_err": float(np.max(np.abs(v.to_numpy() - want)) / np.max(np.abs(want)))}
    del ta, tb
    torch.cuda.empty_cache()
    return out


def run_blas3_section(dev, stream, n_syrk=8192, k_syrk=2048, n=4096):
    """SYRK (n_syrk x k_syrk, lower, beta 0.5), TRSM (n x n lower, n right-hand
    sides) and SYMM (n x n x n) in f64 through the split GEMM, against torch's
    FP64 cuBLAS calls on the same data (A A^T, solve_triangular, matmul); TFLOP/s
    with the conventional counts (SYRK n(n+1)k, TRSM n^2 m, SYMM 2 n^2 m) and
    the relative Frobenius error against the FP64 result."""
    import torch

    import rstsr_gb300 as rt

    out = {}
    rng = np.random.default_rng(0)
    a = rng.standard_normal((n_syrk, k_syrk))
    c = rng.standard_normal((n_syrk, n_syrk))
    ta, tc = rt.asarray(a, dev), rt.asarray(c, dev)
    ga = torch.from_numpy(a).cuda()
    rt.syrk(ta, tc, "L", "N", 1.0, 0.5)
    sec = _time_events(stream, lambda: rt.syrk(ta, tc, "L", "N", 1.0, 0.0), 3)
    sec_t = _time_events(stream, lambda: ga @ ga.T, 1)
    w = rt.empty((n_syrk, n_syrk), np.float64, dev)
    rt.syrk(ta, w, "L", "N", 1.0, 0.0)
    ref = torch.tril(ga @ ga.T)
    err = (torch.linalg.norm(torch.tril(torch.as_tensor(w.to_numpy()).cuda()) - ref) / torch.linalg.norm(ref)).item()
    fl = float(n_syrk) * (n_syrk + 1) * k_syrk
    out["syrk_f64"] = {"n": n_syrk, "k": k_syrk, "tflops": round(fl / sec / 1e12, 2), "ms": round(sec * 1e3, 3),
                       "torch_fp64_tflops": round(fl / sec_t / 1e12, 3), "rel_err_frobenius": err}
    del ta, tc, ga, w, ref
    torch.cuda.empty_cache()
    L = np.tril(rng.standard_normal((n, n)) * 0.02) + np.eye(n) * 2.0
    B = rng.standard_normal((n, n))
    tL, tB = rt.asarray(L, dev), rt.asarray(B, dev)
    gL, gB = torch.from_numpy(L).cuda(), torch.from_numpy(B).cuda()
    work = rt.empty((n, n), np.float64, dev)

    def solve():
        rt.assign(work, tB)
        rt.trsm(tL, work, "L", "L", "N", "N")

    solve()
    sec = _time_events(stream, solve, 3)
    sec_t = _time_events(stream, lambda: torch.linalg.solve_triangular(gL, gB, upper=False), 1)
    ref = torch.linalg.solve_triangular(gL, gB, upper=False)
    err = (torch.linalg.norm(torch.as_tensor(work.to_numpy()).cuda() - ref) / torch.linalg.norm(ref)).item()
    fl = float(n) * n * n
    out["trsm_f64"] = {"m": n, "n": n, "tflops": round(fl / sec / 1e12, 2), "ms": round(sec * 1e3, 3),
                       "torch_fp64_tflops": round(fl / sec_t / 1e12, 3), "rel_err_frobenius": err,
                       "note": "includes the copy of B into the work matrix"}
    S = rng.standard_normal((n, n))
    S = (S + S.T) / 2
    tS = rt.asarray(S, dev)
    tC = rt.empty((n, n), np.float64, dev)
    gS = torch.from_numpy(S).cuda()
    rt.symm(tS, tB, tC, "L", "L")
    sec = _time_events(stream, lambda: rt.symm(tS, tB, tC, "L", "L"), 3)
    sec_t = _time_events(stream, lambda: gS @ gB, 1)
    ref = gS @ gB
    err = (torch.linalg.norm(torch.as_tensor(tC.to_numpy()).cuda() - ref) / torch.linalg.norm(ref)).item()
    fl = 2.0 * n * n * n
    out["symm_f64"] = {"m": n, "n": n, "tflops": round(fl / sec / 1e12, 2), "ms": round(sec * 1e3, 3),
                       "torch_fp64_tflops": round(fl / sec_t / 1e12, 3), "rel_err_frobenius": err}
    del tL, tB, gL, gB, work, tS, tC, gS, ref
    torch.cuda.empty_cache()
    return out


def run_contraction_only(args):
    """Only the contraction section (profiling)."""
    import torch

    import rstsr_gb300 as rt

    dev = rt.DeviceCuda(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    dev.set_stream(stream.cuda_stream)
    res = run_contraction_section(dev, stream, P=args.ein_p)
    res.update(run_blas3_section(dev, stream))
    return {"section": "contraction", "results": res}


def run_trsm_only(args):
    """Only TRSM (profiling): lower triangle L = tril(N(0, 0.02)) + 2 I of order
    --trsm-n, n right-hand sides B ~ N(0, 1), seed 0; each call copies B into
    the work matrix and solves L X = B in place; CUDA events over --steps calls."""
    import torch

    import rstsr_gb300 as rt

    dev = rt.DeviceCuda(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    dev.set_stream(stream.cuda_stream)
    n = args.trsm_n
    rng = np.random.default_rng(0)
    L = np.tril(rng.standard_normal((n, n)) * 0.02) + np.eye(n) * 2.0
    B = rng.standard_normal((n, n))
    tL, tB = rt.asarray(L, dev), rt.asarray(B, dev)
    work = rt.empty((n, n), np.float64, dev)

    def solve():
        rt.assign(work, tB)
        rt.trsm(tL, work, "L", "L", "N", "N")

    for _ in range(max(args.warmup - 1, 0)):
        solve()
    sec = _time_events(stream, solve, max(args.steps, 1))
    return {"section": "trsm", "n": n, "ms": round(sec * 1e3, 3), "tflops": round(float(n) ** 3 / sec / 1e12, 2)}


def run_per_case_only(args):
    """Per-case device time of every operation of the strided workload (each
    call timed alone with CUDA events, the cases cycled so that every input is
    cold: 268 MB f64 / 134 MB f32 operands, nine rounds, median), as a fraction
    of the measured HBM copy rate; and torch's own reductions and copy on
    C-contiguous inputs of the same bytes for comparison."""
    import torch

    import rstsr_gb300 as rt

    dev = rt.DeviceCuda(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    dev.set_stream(stream.cuda_stream)
    try:
        peak = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        peak = 6800.0
    dts = [d for d in args.dtypes.split(",") if d] or None
    lays = [x for x in args.layouts.split(",") if x] or None
    wl = Workload(dev, rt.lib(), seed=0, dtypes=dts, layouts=lays)
    ops = ("to_contig", "fma", "sum", "argmax")
    for c in wl.cases:
        for op in ops:
            wl.run_op(c, op)
    torch.cuda.synchronize()
    ev = {}
    for _ in range(9):
        for op in ops:
            for c in wl.cases:
                if not c["bytes"][op]:
                    continue
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                wl.run_op(c, op)
                e1.record(stream)
                ev.setdefault((c["dname"], c["kind"], op), []).append((e0, e1))
    torch.cuda.synchronize()
    cases = {}
    for (d, k, op), pairs in sorted(ev.items()):
        ms = sorted(a.elapsed_time(b) for a, b in pairs)[len(pairs) // 2]
        c = next(x for x in wl.cases if x["dname"] == d and x["kind"] == k)
        cases[f"{d}/{k}/{op}"] = {"us": round(ms * 1e3, 1),
                                  "frac_hbm": round(c["bytes"][op] / (ms * 1e-3) / 1e9 / peak, 3)}
    del wl
    torch_res = {}
    for dname, dt in DTYPES:
        if dts and dname not in dts:
            continue
        tdt = {"f64": torch.float64, "f32": torch.float32, "i32": torch.int32}[dname]
        if tdt.is_floating_point:
            x = torch.rand(N, device="cuda", dtype=tdt) * 2 - 1
        else:
            x = torch.randint(-1000, 1001, (N,), device="cuda", dtype=tdt)
        nb = N * x.element_size()
        calls = {"sum(1,3)": (lambda: x.view(SHAPE).sum(dim=(1, 3)), nb),
                 "argmax(-1)": (lambda: x.view(SHAPE).argmax(dim=-1), nb),
                 "copy": (lambda: x.clone(), 2 * nb)}
        for name, (fn, b) in calls.items():
            for _ in range(3):
                fn()
            sec = _time_events(stream, fn, 9)
            torch_res[f"{dname}/c/{name}"] = {"us": round(sec * 1e6, 1), "frac_hbm": round(b / sec / 1e9 / peak, 3)}
        del x
    return {"section": "per_case", "peak_gbs": peak, "cases": cases, "torch": torch_res}


def run_c4_only(args):
    """Only the f32 three-term split GEMM (profiling): A [m, k] and B [k, n]
    (--c4-shape, else m = n = k = --c4-n) uniform(-1, 1) scaled by
    2^U(-8, 8), seed 0, C = A B in f32; with
    --c4-tune the project's autotuner picks the tile configuration first.
    CUDA events over --steps calls after --warmup."""
    import torch

    import rstsr_gb300 as rt

    dev = rt.DeviceCuda(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    dev.set_stream(stream.cuda_stream)
    m, n, k = (int(x) for x in args.c4_shape.split(",")) if args.c4_shape else (args.c4_n,) * 3
    rng = np.random.default_rng(0)
    a = (rng.uniform(-1, 1, (m, k)) * 2.0 ** rng.uniform(-8, 8, (m, k))).astype(np.float32)
    b = (rng.uniform(-1, 1, (k, n)) * 2.0 ** rng.uniform(-8, 8, (k, n))).astype(np.float32)
    ta, tb = rt.asarray(a, dev), rt.asarray(b, dev)
    c = rt.empty((m, n), np.float32, dev)
    res = {"section": "c4", "shape": [m, n, k]}
    if args.c4_tune:
        code = rt.autotune_gemm(dev, np.float32, m, n, k)
        res["tuned_config"] = {"k_tile": code & 255, "group": code >> 8}
    for _ in range(max(args.warmup - 1, 0)):
        rt.matmul_into(c, ta, tb)
    sec = _time_events(stream, lambda: rt.matmul_into(c, ta, tb), max(args.steps, 1))
    res.update({"ms": round(sec * 1e3, 3), "tflops": round(2.0 * m * n * k / sec / 1e12, 2)})
    ref = torch.from_numpy(a).cuda().double() @ torch.from_numpy(b).cuda().double()
    got = torch.as_tensor(c.to_numpy()).cuda().double()
    res["rel_err_vs_fp64"] = (torch.linalg.norm(got - ref) / torch.linalg.norm(ref)).item()
    return res


def run_batched_only(args):
    """Only the batched / grouped GEMM section (profiling)."""
    import torch

    import rstsr_gb300 as rt

    dev = rt.DeviceCuda(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    dev.set_stream(stream.cuda_stream)
    return {"section": "batched", "results": run_batched_section(dev, stream)}


def run_tri_index_only(args):
    """Only the packed-triangle / index-selection section (profiling)."""
    import torch

    import rstsr_gb300 as rt

    dev = rt.DeviceCuda(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    dev.set_stream(stream.cuda_stream)
    res = run_tri_index_section(dev, stream, n=args.tri_n, batch=args.tri_batch, rows=args.sel_rows,
                                cols=args.sel_cols)
    return {"section": "tri_index", "results": res}


def run_e2e(wl, dev, stream, args, world):
    """Same step with host buffers, through the C ABI's host-transfer entry
    points: every input copied in (rstsr_cuda_memcpy_h2d_async) and every
    result copied out (rstsr_cuda_memcpy_d2h_async) inside the timed region,
    which ends when the last result is on the host. Two host-memory kinds:
    page-locked buffers (one stream-ordered copy each; copies in, compute and
    copies out of successive cases overlap on three streams) and pageable
    numpy buffers, what a Rust Vec<T> is (chunked staging through the
    context's page-locked ring; the host waits for each result)."""
    import torch

    lib = wl.lib
    n = len(wl.cases)

    def outs_of(c, alloc):
        return {k: alloc(b) for k, b in (("perm", c["out_perm"].size * c["esize"]), ("d", wl_bytes(c["d"])),
                                         ("s", wl_bytes(c["sum_out"])), ("g", wl_bytes(c["arg_out"])))}

    pinned, pageable = [], []
    for c in wl.cases:
        pin = lambda b: torch.empty(b, dtype=torch.uint8).pin_memory()
        pinned.append(([torch.from_numpy(np.ascontiguousarray(x)).pin_memory() for x in (c["ha"], c["hb"], c["hc"])],
                       outs_of(c, pin)))
        pageable.append(([np.ascontiguousarray(x) for x in (c["ha"], c["hb"], c["hc"])],
                         outs_of(c, lambda b: np.empty(b, dtype=np.uint8))))

    def addr(x):
        return x.data_ptr() if isinstance(x, torch.Tensor) else x.ctypes.data

    def nbytes(x):
        return x.numel() * x.element_size() if isinstance(x, torch.Tensor) else x.nbytes

    # three streams: inputs in, compute, results out; the context's stream is
    # switched per phase (rstsr_cuda_ctx_set_stream), events order the phases
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    s_comp = stream
    ev_in = [torch.cuda.Event() for _ in range(n)]
    ev_comp = [torch.cuda.Event() for _ in range(n)]

    def step(bufs):
        h2d = d2h = 0
        for i, (c, (ins, outs)) in enumerate(zip(wl.cases, bufs)):
            dev.set_stream(s_in.cuda_stream)
            for host, t in zip(ins, (c["a"], c["b"], c["c"])):
                rc = lib.rstsr_cuda_memcpy_h2d_async(dev.ctx, C.c_void_p(t.ptr), C.c_void_p(addr(host)),
                                                     C.c_size_t(nbytes(host)))
                assert rc == 0, lib.rstsr_cuda_last_error().decode()
                h2d += nbytes(host)
            ev_in[i].record(s_in)
            s_comp.wait_event(ev_in[i])
            dev.set_stream(s_comp.cuda_stream)
            for op in ("to_contig", "fma", "sum", "argmax"):
                wl.run_op(c, op)
            ev_comp[i].record(s_comp)
            s_out.wait_event(ev_comp[i])
            dev.set_stream(s_out.cuda_stream)
            for key, t in (("perm", c["out_perm"] if c["copy"] else None), ("d", c["d"]), ("s", c["sum_out"]),
                           ("g", c["arg_out"])):
                if t is None:
                    continue
                rc = lib.rstsr_cuda_memcpy_d2h_async(dev.ctx, C.c_void_p(addr(outs[key])), C.c_void_p(t.ptr),
                                                     C.c_size_t(nbytes(outs[key])))
                assert rc == 0, lib.rstsr_cuda_last_error().decode()
                d2h += nbytes(outs[key])
        dev.set_stream(s_comp.cuda_stream)
        return h2d, d2h

    steps = max(10, min(args.steps, 20))
    res = {}
    for name, bufs in (("pinned", pinned), ("pageable", pageable)):
        for _ in range(max(1, args.warmup // 2)):
            step(bufs)
            torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            h2d, d2h = step(bufs)
            torch.cuda.synchronize()  # a step ends when its last result is on the host
        rate, t = replicas.whole_job_rate(wl.total_bytes(), (time.perf_counter() - t0) / steps, "cuda")
        res[name] = {"value": round(rate / 1e9, 1), "unit": "GB/s", "h2d_bytes_per_step": int(h2d),
                     "d2h_bytes_per_step": int(d2h), "ms_per_step": round(t * 1e3, 3), "steps": steps}
    dev.set_stream(stream.cuda_stream)
    out = dict(res["pinned"])
    out["host_memory"] = "page-locked (pinned); wall clock over the timed steps"
    out["pageable"] = {k: res["pageable"][k] for k in ("value", "ms_per_step")}
    return out


def wl_bytes(t):
    lo, hi = t.offset, t.offset + 1
    for d, s in zip(t.shape, t.stride):
        if s > 0:
            hi += s * (d - 1)
        else:
            lo += s * (d - 1)
    return (hi - lo) * t.itemsize


# ------------------------------------------------------------ CPU legs


def host_cases(seed=0, src=None, batch=32):
    """Host inputs of every (dtype, layout) case of the step, restricted to
    the leading `batch` of the 32 indices of axis 0 (a view with the full
    tensor's strides). `src` is the GPU workload, whose own host buffers are
    then used; otherwise the buffers are generated with the workload's seeds."""
    shape = (batch,) + SHAPE[1:]
    out = []
    for di, (dname, dt) in enumerate(DTYPES):
        for li, kind in enumerate(LAYOUTS):
            if src is not None:
                c = next((x for x in src.cases if x["dname"] == dname and x["kind"] == kind), None)
                if c is None:
                    continue
                ha, hb, hc = c["ha"], c["hb"], c["hc"]
            else:
                blen, _, _ = layout_of(kind, SHAPE)
                ha = host_data(dt, blen, seed + 10 * di + li)
                hb = host_data(dt, blen, seed + 1000 + 10 * di + li)
                hc = host_data(dt, int(np.prod(CSHAPE)), seed + 100 + di)
            _, stride, off = layout_of(kind, SHAPE)
            out.append(dict(dname=dname, kind=kind, dt=dt, esize=np.dtype(dt).itemsize, shape=shape, stride=stride,
                            off=off, ha=ha, hb=hb, hc=hc))
    return out


def cpu_step(cases, nthreads, reps=1, keep=False):
    """The step's operations on the CPU oracle (OpenMP restatement of the
    reference's rayon kernels) over `cases`, each case's operations timed
    `reps` times. The reference's two passes for a*b+c: tmp = a*b in the
    binary-op layout, then tmp += c. Returns (seconds, algorithmic bytes,
    outputs of the last repetition per case if `keep`)."""
    from oracle import layout as OL
    from oracle import oracle as O

    tot_t, tot_b, outs = 0.0, 0, []
    for cs in cases:
        shape, stride, off, dt = cs["shape"], cs["stride"], cs["off"], cs["dt"]
        n = int(np.prod(shape))
        a = O.Strided(cs["ha"], shape, stride, off)
        b = O.Strided(cs["hb"], shape, stride, off)
        cst = O.Strided(cs["hc"], shape, (0, CSHAPE[3], 0, 1), 0)
        pshape, pstride = permuted_view(shape, stride)
        lab = OL.layout_for_binary_op((shape, stride, off), (shape, stride, off))
        so_l = OL.reduce_output_layout((shape, stride, off), [1, 3])
        go_l = OL.reduce_output_layout((shape, stride, off), [3])
        res = None
        for _ in range(reps):
            t0 = time.perf_counter()
            dst = None
            if cs["kind"] != "perm":
                dst = O.empty_strided(pshape, c_stride(pshape), dt)
                O.assign_arbitrary(dst, O.Strided(cs["ha"], pshape, pstride, off), 0, nthreads)
            tmp = O.empty_strided(lab[0], lab[1], dt)
            O.binary("mul", tmp, a, b, nthreads)
            O.binary("add", tmp, tmp, cst, nthreads)
            so = O.empty_strided(so_l[0], so_l[1], dt)
            O.reduce_axes("sum", a, [1, 3], so, nthreads)
            go = O.empty_strided(go_l[0], go_l[1], np.uint64)
            O.argreduce_axes(True, a, [3], go, nthreads)
            tot_t += time.perf_counter() - t0
            tot_b += op_bytes_n(cs["esize"], cs["kind"], n, shape)
            res = (dst, tmp, so, go)
        if keep:
            outs.append(res)
    return tot_t, tot_b, outs


def op_bytes_n(esize, kind, n, shape):
    copy = 2 * n * esize if kind != "perm" else 0
    return (copy + (3 * n + int(np.prod(CSHAPE))) * esize + (n + shape[0] * shape[2]) * esize
            + n * esize + shape[0] * shape[1] * shape[2] * 8)


def check_outputs(wl, cases, outs):
    """Compare the GPU outputs of the timed step (leading `batch` slabs of
    every case) with the oracle's outputs on the same host data: copies, the
    fused a*b+c and argmax bit-exact, sums within 1e-13 (f64) / 1e-5 (f32)
    normwise, integers exact."""
    bad, worst = [], {}
    for cs, (dst, tmp, so, go) in zip(cases, outs):
        c = next(x for x in wl.cases if x["dname"] == cs["dname"] and x["kind"] == cs["kind"])
        lead = (slice(0, cs["shape"][0]),)
        name = f"{cs['dname']}/{cs['kind']}"
        if dst is not None and not np.array_equal(c["out_perm"].i(lead).to_numpy(), dst.values()):
            bad.append(name + "/to_contig")
        if not np.array_equal(c["d"].i(lead).to_numpy(), tmp.values()):
            bad.append(name + "/fma")
        got, want = c["sum_out"].i(lead).to_numpy(), so.values()
        if np.dtype(cs["dt"]).kind == "i":
            if not np.array_equal(got, want):
                bad.append(name + "/sum")
        else:
            err = float(np.max(np.abs(got.astype(np.float64) - want)) / max(float(np.max(np.abs(want))), 1e-300))
            worst[cs["dname"]] = max(worst.get(cs["dname"], 0.0), err)
            if err > (1e-13 if cs["dt"] == np.float64 else 1e-5):
                bad.append(name + "/sum")
        if not np.array_equal(c["arg_out"].i(lead).to_numpy(), go.values()):
            bad.append(name + "/argmax")
    return {"ok": not bad, "mismatches": bad,
            "checked": f"every output of the timed step on the leading {cases[0]['shape'][0]} of 32 slabs "
                       "of every case against the oracle (copies, a*b+c, argmax and integer sums bit-exact)",
            "sum_max_normwise_err": {k: float(f"{v:.3g}") for k, v in worst.items()}}


def cpu_baseline(args, wl=None):
    """The oracle on all host cores on a bounded sample of the step (the
    leading --cpu-batch of 32 slabs, the GPU workload's own host data), its
    operations repeated until about --cpu-seconds of CPU work is timed. With
    the GPU workload given, the outputs of that sample also check the GPU's."""
    from oracle import oracle as O

    nth = O.max_threads()
    cases = host_cases(src=wl, batch=args.cpu_batch)
    t, b, outs = cpu_step(cases, nth, keep=wl is not None)  # one pass sizes the repeat count
    parity = check_outputs(wl, cases, outs) if wl is not None else None
    del outs
    reps = max(1, min(200, math.ceil(args.cpu_seconds / max(t, 1e-3))))
    if reps > 1:
        t, b, _ = cpu_step(cases, nth, reps=reps)
    res = {"value": round(b / t / 1e9, 2), "unit": "GB/s", "cores": nth, "kind": "port",
           "sample": f"the step at leading extent {args.cpu_batch} of 32 (all dtypes and layouts), each case's "
                     f"operations timed {reps} times: {b / 1e9:.2f} GB in {t:.2f} s"}
    return res, parity


def run_reference(args):
    """The reference arm: the OpenMP restatement of rstsr's rayon kernels on
    every host core, on the full workload (all 32 slabs, every dtype and
    layout); inputs generated once, each step one pass of the operations."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    from oracle import oracle as O

    nth = O.max_threads()
    cases = host_cases(batch=args.ref_batch)
    for _ in range(args.warmup):
        cpu_step(cases, nth)
    tt, bb = 0.0, 0
    for _ in range(args.steps):
        t, b, _ = cpu_step(cases, nth)
        tt += t
        bb += b
    value = bb / tt / 1e9
    what = "the full workload, all 32 slabs" if args.ref_batch == 32 else f"leading extent {args.ref_batch} of 32"
    sample = f"each step: {what}, all dtypes and layouts ({bb / args.steps / 1e9:.2f} GB)"
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": round(value, 2),
        "unit": "GB/s",
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(tt / args.steps * 1e3, 2),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64,f32,i32",
        "data": "synthetic (seeded uniform; i32 uniform in [-1000,1000])",
        "config": {"workload": WORKLOAD, "parallelism": "host cores"},
        "cpu_baseline": {"value": round(value, 2), "unit": "GB/s", "cores": nth, "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 2), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-gemm", action="store_true")
    ap.add_argument("--cpu-batch", type=int, default=4, help="leading slabs of the cpu_baseline sample")
    ap.add_argument("--ref-batch", type=int, default=32,
                    help="leading slabs of the reference arm's step (32: the full workload)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="CPU work the cpu_baseline sample is sized to (the operations repeated)")
    # restrict the workload (profiling a small case): comma-separated subsets
    ap.add_argument("--dtypes", default="", help="subset of f64,f32,i32")
    ap.add_argument("--layouts", default="", help="subset of c,f,perm,slice")
    ap.add_argument("--rate-n", type=int, default=8192, help="matrix order for --only rates")
    ap.add_argument("--trsm-n", type=int, default=4096, help="order (and right-hand sides) for --only trsm")
    ap.add_argument("--only", default="",
                    choices=["", "c3", "c4", "tri_index", "contraction", "rates", "batched", "trsm", "per_case"],
                    help="c3: only the Ozaki contraction; tri_index: only pack/unpack_tri and index_select; "
                         "contraction: only einsum / vecdot; rates: INT8 / BF16 / FP64 tensor rates; batched: only C5; "
                         "c4: only the f32 split GEMM (--c4-n, --c4-tune); trsm: only TRSM; per_case: each operation of the strided workload per (dtype, layout), "
                         "with torch's reductions on the same bytes")
    ap.add_argument("--ein-p", type=int, default=1000, help="P of the 3-index transform for --only contraction")
    ap.add_argument("--c4-n", type=int, default=8192, help="order of the f32 product for --only c4")
    ap.add_argument("--c4-shape", default="", help="M,N,K of the f32 product for --only c4 (overrides --c4-n)")
    ap.add_argument("--c4-tune", action="store_true", help="autotune the tile configuration first (--only c4)")
    ap.add_argument("--c3-cols", type=int, default=15000, help="columns of Bm for --only c3")
    ap.add_argument("--tri-n", type=int, default=2048, help="matrix order for --only tri_index")
    ap.add_argument("--tri-batch", type=int, default=32, help="matrices for --only tri_index")
    ap.add_argument("--sel-rows", type=int, default=16384, help="rows of the index_select source")
    ap.add_argument("--sel-cols", type=int, default=8192, help="columns of the index_select source")
    args = ap.parse_args()
    if args.only == "c3":
        res = run_c3_only(args)
    elif args.only == "rates":
        res = run_rates(args)
    elif args.only == "batched":
        res = run_batched_only(args)
    elif args.only == "trsm":
        res = run_trsm_only(args)
    elif args.only == "per_case":
        res = run_per_case_only(args)
    elif args.only == "c4":
        res = run_c4_only(args)
    elif args.only == "tri_index":
        res = run_tri_index_only(args)
    elif args.only == "contraction":
        res = run_contraction_only(args)
    elif args.impl == "reference":
        res = run_reference(args)
    else:
        res = run_gpu(args)
    if res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
