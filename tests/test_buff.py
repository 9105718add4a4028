"""The observable buffer (lbm_gb300.buff: preallocated histories instead of
np.append at every call) against the reference's buff (lbm/src/utils/buff.py:8-77)
on the golden series of tests/golden/buff.npz: the same moving averages,
growth rates and convergence flag at every iteration, bit for bit.  No GPU."""
import os
import sys

import numpy as np

from lbm_gb300.buff import buff

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_golden import BUFF_ARGS  # noqa: E402


def test_buff_matches_reference_series():
    d = np.load(os.path.join(HERE, "golden", "buff.npz"))
    b = buff("drag", BUFF_ARGS["dt"], BUFF_ARGS["obs_cv_ct"], BUFF_ARGS["obs_cv_nb"], ".")
    obs, growth, cv = [], [], []
    for v in d["buff"][2:]:
        b.add(v)
        o, g = b.mv_avg()
        obs.append(o)
        growth.append(g)
        cv.append(int(b.obs_cv))
    assert np.array_equal(np.array(obs), d["obs"])
    assert np.array_equal(np.array(growth), d["growth"])
    assert np.array_equal(np.array(cv), d["cv"])
    assert d["cv"].any() and not d["cv"][:100].any()   # the flag flips during the run
    for k, ref in (("buff", d["buff"]), ("avg1_buff", d["avg1"]), ("avg2_buff", d["avg2"]),
                   ("avg3_buff", d["avg3"])):
        assert np.array_equal(getattr(b, k), ref), k
    assert b.f_avg() == float(d["f_avg"])
