"""A lone transform on a thread-block cluster (the latency path of the plain small case).

One binary64 transform of N <= 4096 points on a contiguous line runs on a cluster of up to 8
CTAs that keep the array in every CTA's shared memory and exchange each pass's outputs through
distributed shared memory.  Its passes are the reference codelets, so every result equals the
oracle's refTransform with the plan's radices bit for bit: out of place and in place, both
directions, with the radices of least latency the planner picks for a lone transform and with
explicit radix sequences, and with an output scale."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
import oracle as O  # noqa: E402

SIZES = [2, 3, 8, 16, 60, 64, 210, 360, 1000, 1024, 1080, 2048, 3003, 4096]


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


@pytest.mark.parametrize("sign", [-1, 1])
@pytest.mark.parametrize("n", SIZES)
def test_lone_transform_bitexact(n, sign):
    x = O.uniform_complex((1, n), seed=n + sign)
    plan = lfg.plan_1d(n, sign, 1)
    assert plan.info().cluster_ctas >= 1, n
    xd = torch.from_numpy(x).cuda()
    y = plan.execute(xd)
    z = xd.clone()
    plan.execute(z, z)                               # in place
    torch.cuda.synchronize()
    ref = O.ref_transform(sign < 0, n, plan.radices, x)
    assert np.array_equal(_bits(y.cpu().numpy()), _bits(ref)), (n, plan.radices)
    assert torch.equal(z.view(torch.float64), y.view(torch.float64))


@pytest.mark.parametrize("n,rs", [(1024, [16, 16, 4]), (1024, [2] * 10), (1024, [4] * 5),
                                  (4096, [16, 16, 16]), (360, [8, 9, 5]), (2048, [2, 16, 8, 8])])
def test_explicit_radices_on_the_cluster(n, rs):
    x = O.uniform_complex((1, n), seed=7)
    plan = lfg.plan_1d(n, -1, 1, radices=rs)
    assert plan.info().cluster_ctas >= 1
    y = plan.execute(torch.from_numpy(x).cuda())
    torch.cuda.synchronize()
    assert np.array_equal(_bits(y.cpu().numpy()), _bits(O.ref_transform(True, n, rs, x)))


def test_scaled_output():
    n = 1024
    x = O.uniform_complex((1, n), seed=3)
    plan = lfg.plan_1d(n, 1, 1)
    xd = torch.from_numpy(x).cuda()
    y = plan.execute(xd)
    plan.set_scale(0.25)
    ys = plan.execute(xd)
    torch.cuda.synchronize()
    assert torch.equal(ys, y * 0.25)                 # a power of two: exact
