"""The tensor-core operand layouts and descriptors of this library (tcgen05
MMA, bf16 operands in shared memory, FP32 accumulation in tensor memory)
against exact host products, and the integer exactness of the FP32
accumulation that the split-precision exchange relies on.

Integer operands of magnitude <= 256 are exact in bf16, and sums of their
products are exact in FP32 while they stay below 2^24; the checks below are
equalities, not tolerances."""
import numpy as np
import pytest

import helfem_gb300 as hg
from gpu_util import torch_cuda

pytestmark = pytest.mark.gpu


def _ints(rng, shape, lo, hi):
    return rng.integers(lo, hi + 1, size=shape).astype(np.float32)


@pytest.mark.parametrize("N,ksteps,a_mn,b_mn", [(16, 1, 0, 0), (96, 1, 0, 0), (256, 2, 0, 0), (16, 1, 1, 0),
                                                (112, 3, 1, 0), (32, 1, 0, 1), (64, 2, 1, 1)])
def test_tc_layouts_exact(N, ksteps, a_mn, b_mn):
    torch_cuda()
    rng = np.random.default_rng(N * 10 + ksteps + 3 * a_mn + 7 * b_mn)
    A = _ints(rng, (128, 16 * ksteps), -128, 128)
    B = _ints(rng, (N, 16 * ksteps), -128, 128)
    ref = A.astype(np.int64) @ B.astype(np.int64).T
    D = hg.tc_selftest(A, B, a_mn_major=bool(a_mn), b_mn_major=bool(b_mn))
    bad = int(np.count_nonzero(D.astype(np.int64) != ref))
    if bad:  # which stride convention would have matched (diagnostic only)
        S = hg.tc_selftest(A, B, a_mn_major=bool(a_mn), b_mn_major=bool(b_mn), swap_offsets=True)
        swapped = int(np.count_nonzero(S.astype(np.int64) != ref))
        pytest.fail(f"{bad} of {D.size} entries differ (with the strides exchanged: {swapped})")


def test_tc_fp32_accumulation_is_exact_for_integer_sums():
    """Eight K steps of digit products (|a|, |b| <= 256) whose exact sums reach
    a few times 2^21: the tensor-memory accumulation must not round."""
    torch_cuda()
    rng = np.random.default_rng(5)
    A = _ints(rng, (128, 128), 200, 256)
    B = _ints(rng, (256, 128), 200, 256)
    A[::3] *= -1
    ref = A.astype(np.int64) @ B.astype(np.int64).T
    assert np.abs(ref).max() > 2 ** 22 and np.abs(ref).max() < 2 ** 24
    D = hg.tc_selftest(A, B)
    assert np.array_equal(D.astype(np.int64), ref)


def test_tc_peak_runs():
    torch_cuda()
    r = hg.tc_peak(2, 2048)
    print(f"dense bf16 tcgen05 rate: {r['tflops']:.1f} TFLOP/s ({r['ms']:.3f} ms)")
    assert r["tflops"] > 100.0
