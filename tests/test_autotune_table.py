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
