"""Tuning cache on the GPU: a second LFG_MEASURE plan of the same problem takes the stored
schedule without timing candidates, and a stored entry that names an invalid schedule is
ignored (the problem is measured again).  Timings are counted through LFG_PLAN_LOG, which
receives one line per timed candidate."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
import oracle as O  # noqa: E402


def _lines(p):
    return sum(1 for _ in open(p)) if os.path.exists(p) else 0


def test_second_measured_plan_uses_the_cache(tmp_path, monkeypatch):
    log = tmp_path / "plan.log"
    monkeypatch.setenv("LFG_PLAN_LOG", str(log))
    lfg.wisdom_forget()
    p1 = lfg.plan_1d(1000, -1, 64, measure=True)
    timed = _lines(log)
    assert timed > 0 and lfg.wisdom_count() == 1
    p2 = lfg.plan_1d(1000, -1, 64, measure=True)
    assert _lines(log) == timed                       # nothing timed the second time
    assert p2.radices == p1.radices
    x = O.uniform_complex((64, 1000), seed=4)
    xd = torch.from_numpy(x).cuda()
    y1, y2 = p1.execute(xd), p2.execute(xd)
    torch.cuda.synchronize()
    assert torch.equal(y1.view(torch.float64), y2.view(torch.float64))
    ref = O.ref_transform(True, 1000, p2.radices, x)
    assert np.array_equal(y2.cpu().numpy().view(np.uint64), ref.view(np.uint64))

    # ragged batches, and the file carries the table to a fresh table
    sizes = lfg.ragged_sizes(256, seed=3)
    r1 = lfg.plan_ragged(sizes, -1, measure=True)
    timed = _lines(log)
    f = tmp_path / "w"
    lfg.wisdom_export(str(f))
    lfg.wisdom_forget()
    lfg.wisdom_import(str(f))
    assert lfg.wisdom_count() == 2
    r2 = lfg.plan_ragged(sizes, -1, measure=True)
    assert _lines(log) == timed
    i1, i2 = r1.info(), r2.info()
    assert (i1.block_shape, i1.tile_target, i1.single_max) == (i2.block_shape, i2.tile_target, i2.single_max)
    lfg.wisdom_forget()


def test_invalid_entry_is_measured_again(tmp_path, monkeypatch):
    log = tmp_path / "plan.log"
    monkeypatch.setenv("LFG_PLAN_LOG", str(log))
    lfg.wisdom_forget()
    f = tmp_path / "bad"
    lines = 16384   # the autotuner's scratch batch for n = 1024 (256 MB cap)
    f.write_text(f"c2c n=1024 precision=0 fwd=1 lines={lines}\tradices=16,16,3;single=2048;tile=2048\n")
    lfg.wisdom_import(str(f))
    p = lfg.plan_1d(1024, -1, 1 << 14, measure=True)
    assert _lines(log) > 0                            # 16*16*3 != 1024: re-measured
    r = 1
    for v in p.radices:
        r *= v
    assert r == 1024
    lfg.wisdom_forget()
