"""Host-side pieces of bench.py's legs (no GPU): the multi-echo leg's
schedule."""
import math
import os
import sys

import numpy as np


def _bench():
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    return bench


def test_cpmg_schedule():
    """A 90 about y at step 0, then a 180 about x every CPMG_ECHO steps from
    CPMG_ECHO / 2: the timed window [S, 3S) holds 2S / CPMG_ECHO pulse steps
    of one pulse each, all fixed-angle (so every step stays on the fast
    path), under the gradient CPMG_G along z on every step run."""
    b = _bench()
    S = b.STEPS_PER_ITER
    wave, rf = b.cpmg_schedule(3 * S)
    assert wave.shape == (3 * S + 16, 3)
    assert np.all(wave[:, 2] == b.CPMG_G) and not np.any(wave[:, :2])
    assert rf[0] == (0, 2, 0.5 * math.pi, (0.0, 1.0, 0.0))
    steps = [q for q, *_ in rf[1:]]
    assert steps[0] == b.CPMG_ECHO // 2 and np.all(np.diff(steps) == b.CPMG_ECHO)
    assert all(f == 2 and p == math.pi and ax == (1.0, 0.0, 0.0) for _, f, p, ax in rf[1:])
    timed = [q for q, *_ in rf if S <= q < 3 * S]
    assert len(timed) == len(set(timed)) == 2 * S // b.CPMG_ECHO
