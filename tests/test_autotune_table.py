"""The GEMM autotune table's text format: load, save, reject malformed files
(host-only entry points, no GPU)."""

import pytest

import rstsr_gb300 as rt


def entries(text):
    return sorted(line.split() for line in text.splitlines() if line.strip() and not line.startswith("#"))


def test_load_save_round_trip(built_lib, tmp_path):
    src = tmp_path / "table.txt"
    src.write_text("# comment\nozaki 7 14 14 10 16 16\n\nbf16x3 3 13 13 13 32 8\n")
    rt.autotune_load(src)
    out = tmp_path / "saved.txt"
    rt.autotune_save(out)
    assert entries(out.read_text()) == entries(src.read_text())


@pytest.mark.parametrize(
    "bad",
    ["ozaki 7 14 14 10 24 16\n", "ozaki 9 14 14 10 16 16\n", "int8 7 14 14 10 16 16\n", "ozaki 7 14 14\n",
     "bf16x3 3 13 13 13 32 0\n"],
)
def test_malformed_file_is_rejected_and_table_kept(built_lib, tmp_path, bad):
    good = tmp_path / "good.txt"
    good.write_text("ozaki 6 10 10 10 32 4\n")
    rt.autotune_load(good)
    bad_file = tmp_path / "bad.txt"
    bad_file.write_text(bad)
    with pytest.raises(rt.RstsrError):
        rt.autotune_load(bad_file)
    out = tmp_path / "after.txt"
    rt.autotune_save(out)
    assert entries(out.read_text()) == [["ozaki", "6", "10", "10", "10", "32", "4"]]


def test_missing_file_is_an_error(built_lib, tmp_path):
    with pytest.raises(rt.RstsrError):
        rt.autotune_load(tmp_path / "does_not_exist.txt")


def _in_child(tmp_path, env_value, body):
    """Run `body` in a fresh interpreter (the environment table loads once per
    process) with RSTSR_CUDA_AUTOTUNE_TABLE set; return its stdout."""
    import os
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    env = dict(os.environ, RSTSR_CUDA_AUTOTUNE_TABLE=str(env_value), PYTHONPATH=str(root))
    script = "import rstsr_gb300 as rt\n" + body
    res = subprocess.run([sys.executable, "-c", script], cwd=root, env=env, capture_output=True, text=True,
                         timeout=120)
    assert res.returncode == 0, res.stderr
    return res.stdout


def test_environment_table_is_loaded_by_the_first_context(built_lib, tmp_path):
    table = tmp_path / "env_table.txt"
    table.write_text("ozaki 7 12 12 9 32 8\nbf16x3 3 11 11 11 16 4\n")
    out = tmp_path / "saved.txt"
    body = (
        "try:\n    rt.DeviceCuda(0)\nexcept rt.RstsrError:\n    pass  # no GPU here: the table loads first\n"
        f"rt.autotune_save({str(out)!r})\n"
    )
    _in_child(tmp_path, table, body)
    assert entries(out.read_text()) == entries(table.read_text())


@pytest.mark.parametrize("content", ["ozaki 7 12 12 9 24 8\n", None])
def test_bad_environment_table_fails_context_creation(built_lib, tmp_path, content):
    table = tmp_path / "env_table.txt"
    if content is not None:
        table.write_text(content)
    body = (
        "for _ in range(2):\n"
        "    try:\n        rt.DeviceCuda(0)\n        print('created')\n"
        "    except rt.RstsrError as e:\n        print(e.kind, str(e))\n"
    )
    lines = _in_child(tmp_path, table, body).splitlines()
    assert len(lines) == 2 and all("RSTSR_CUDA_AUTOTUNE_TABLE" in line for line in lines), lines
    want = "InvalidValue" if content is not None else "RuntimeError"
    assert all(line.startswith(want) for line in lines), lines
