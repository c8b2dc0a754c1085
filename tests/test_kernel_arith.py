"""Host restatements of small exact-arithmetic helpers of the event kernels
(mc-old_gb300/csrc/mc_event_kernels.cuh), checked over their whole input
range.  IEEE single precision with round-to-nearest, as the device
intrinsics (__frcp_rn, __fadd_rn, __fmul_rn) compute it."""
import numpy as np


def div_small(a: int, b: int) -> int:
    """div_small: (int)(((float)a + 0.5f) * rcp_rn((float)b))."""
    r = np.float32(1.0) / np.float32(b)            # correctly rounded reciprocal
    return int(np.float32(np.float32(a) + np.float32(0.5)) * r)


def test_div_small_is_exact_over_its_range():
    # used by the warp-cooperative free-gas sampler: lane / pending count,
    # first hit / pending count and (32 - rank + np - 1) / np
    for b in range(1, 33):
        for a in range(0, 65):
            assert div_small(a, b) == a // b, (a, b)
