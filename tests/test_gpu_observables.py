"""Observables on the device (lbm_mv_avg_chunk through buff.add_chunk, and
the turek app's chunked observables in the fused runner) against the
reference buffer and the per-iteration replay, bit for bit.

Reference: lbm/src/utils/buff.py:35-77 (moving averages and convergence),
lbm/src/app/turek.py:140-162 (drag_lift lines), base_app.py:53-69
(check_stop)."""
import os
import sys

import numpy as np
import pytest

from _cases import GOLDEN, make_case, run_gpu
from lbm_gb300.buff import buff

sys.path.insert(0, GOLDEN)
from make_golden import BUFF_ARGS  # noqa: E402

pytestmark = pytest.mark.gpu


def _split(vals, sizes):
    out, k = [], 0
    for n in sizes:
        out.append(vals[k:k + n])
        k += n
    out.append(vals[k:])
    return out


def test_add_chunk_matches_reference_goldens(cuda):
    """The reference buffer's 3,000-value golden series, fed in uneven
    chunks: every returned average, growth rate and flag, and the histories."""
    d = np.load(os.path.join(GOLDEN, "buff.npz"))
    b = buff("drag", BUFF_ARGS["dt"], BUFF_ARGS["obs_cv_ct"], BUFF_ARGS["obs_cv_nb"], ".")
    obs, growth, cv = [], [], []
    for part in _split(d["buff"][2:], [1, 7, 300, 1200]):
        o, g, c = b.add_chunk(part)
        obs.append(o)
        growth.append(g)
        cv.append(c)
    assert np.array_equal(np.concatenate(obs), d["obs"])
    assert np.array_equal(np.concatenate(growth), d["growth"])
    assert np.array_equal(np.concatenate(cv).astype(int), d["cv"])
    assert b.obs == d["obs"][-1] and b.obs_cv == bool(d["cv"][-1])
    for k, ref in (("buff", d["buff"]), ("avg1_buff", d["avg1"]), ("avg2_buff", d["avg2"]),
                   ("avg3_buff", d["avg3"])):
        got = getattr(b, k)
        bad = np.flatnonzero(got != ref)
        assert len(bad) == 0, (k, bad[:8], got[bad[:8]], ref[bad[:8]])


def test_add_chunk_long_series_matches_host_buffer(cuda):
    """60,000 values (windows of up to 12,000, deep pairwise splits), chunks
    of 5,000, against the host buffer (pinned to the reference goldens by
    test_buff); then the host path continues from the device histories."""
    rng = np.random.default_rng(9)
    vals = 2.0 + 0.3 * np.sin(np.arange(60000) / 37.0) + 1e-2 * rng.standard_normal(60000)
    host = buff("lift", 0.002, 1e-1, 200, ".")
    dev = buff("lift", 0.002, 1e-1, 200, ".")
    h_obs, h_g, h_cv = [], [], []
    for v in vals:
        host.add(v)
        o, g = host.mv_avg()
        h_obs.append(o)
        h_g.append(g)
        h_cv.append(host.obs_cv)
    got = [dev.add_chunk(p) for p in _split(vals, [5000] * 11)]
    assert np.array_equal(np.concatenate([g[0] for g in got]), h_obs)
    assert np.array_equal(np.concatenate([g[1] for g in got]), h_g)
    assert np.array_equal(np.concatenate([g[2] for g in got]), h_cv)
    assert dev.obs_cv_cnt == host.obs_cv_cnt
    for v in (1.5, 2.5):
        host.add(v)
        dev.add(v)
        assert host.mv_avg() == dev.mv_avg()


def _turek(stop):
    app, n0 = make_case("turek24")
    app.stop = stop
    if stop == "obs":
        # converges after ~2,000 iterations (the oracle stops at 2,019)
        app.obs_cv_ct, app.obs_cv_nb = 5e-2, 40
    return app


class _PerIteration:
    """The same app with the per-iteration replay (no chunk hook)."""
    observables_chunk = None


@pytest.mark.parametrize("stop", ["it", "obs"])
def test_turek_chunked_observables_match_per_iteration(cuda, stop):
    """turek 24 (Re 20): the drag_lift file, the stop iteration and the final
    state of the chunked runner equal the per-iteration replay's (chunks of
    128 iterations, so a convergence stop falls inside a chunk)."""
    a = _turek(stop)
    b = _turek(stop)
    b.__class__ = type("turek_per_iteration", (_PerIteration, type(b)), {})
    out_a, _, lat_a = run_gpu(a, fused=True, chunk=128, record=False)
    out_b, _, lat_b = run_gpu(b, fused=True, chunk=128, record=False)
    with open(lat_a.output_dir + "drag_lift") as f:
        lines_a = f.read()
    with open(lat_b.output_dir + "drag_lift") as f:
        lines_b = f.read()
    assert lines_a == lines_b
    n_lines = lines_a.count("\n")
    assert n_lines > 300
    if stop == "obs":
        assert a.drag_buff.obs_cv and a.lift_buff.obs_cv
        assert n_lines < 4000  # converged and stopped
    for k in ("g", "g_up", "rho", "u"):
        assert np.array_equal(out_a[k], out_b[k]), k
    assert a.drag_buff.obs == b.drag_buff.obs and a.lift_buff.obs == b.lift_buff.obs
