"""Tuning cache ("wisdom"): file format round trip and malformed entries (no GPU needed).

lean-fftw re-measures every plan (LeanFFTW/Asm/Planner.lean:209-286); this library keeps the
autotuner's choices in a table that files can carry between processes, as FFTW's wisdom does.
The GPU side (a second measured plan reusing the stored choice) is in test_gpu_wisdom.py.
"""
import lfg


def _entries(path):
    out = {}
    for line in open(path):
        if line.startswith("#") or "\t" not in line:
            continue
        k, v = line.rstrip("\n").split("\t")
        out[k] = v
    return out


def test_import_export_round_trip(tmp_path):
    lfg.wisdom_forget()
    src = tmp_path / "in.wisdom"
    src.write_text("# comment line\n"
                   "c2c n=1024 precision=0 fwd=1 lines=16384\tradices=16,16,4;single=2048;tile=2048\n"
                   "ragged precision=0 fwd=1 count=8 hash=00000000deadbeef\tshape=0;tile=2048;single=2048\n"
                   "no tab on this line\n"
                   "\n")
    lfg.wisdom_import(str(src))
    assert lfg.wisdom_count() == 2
    dst = tmp_path / "out.wisdom"
    lfg.wisdom_export(str(dst))
    assert _entries(dst) == _entries(src)
    # importing the same file again merges (no duplicates)
    lfg.wisdom_import(str(dst))
    assert lfg.wisdom_count() == 2
    lfg.wisdom_forget()
    assert lfg.wisdom_count() == 0


def test_import_missing_file_is_an_error(tmp_path):
    try:
        lfg.wisdom_import(str(tmp_path / "absent.wisdom"))
    except lfg.LfgError:
        return
    raise AssertionError("importing a missing file must fail")
