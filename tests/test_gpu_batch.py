"""Batched lattices: a lattice advanced inside a batch gives the same bits as
the same lattice advanced alone (same per-cell code, its own tables and
scratch), for vectorised (ny % 8 == 0) and scalar tiles, cavities and IBB
channels, FP16-shifted, fixed-point and FP64 storage, and each scheduling
of the batch kernels."""
import numpy as np
import pytest

from lbm_gb300.apps import cavity
from lbm_gb300.batch import Batch, channel_squares, default_config, sweep_apps
from lbm_gb300.run import _finalize_state

pytestmark = pytest.mark.gpu


def _apps():
    out = []
    for n, re in ((64, 300.0), (70, 800.0), (96, 150.0)):
        a = cavity()
        a.L_lbm, a.Re_lbm, a.u_lbm = n, re, 0.1
        a.compute_lbm_parameters()
        a.sigma = 30.0
        out.append(a)
    out.append(channel_squares(64, [(90.0, 30.0, 8.0), (150.0, 20.0, 6.0)], 400.0))
    out.append(channel_squares(50, [(80.0, 25.0, 7.0)], 300.0))
    for a in out[3:]:
        a.sigma = 30.0
    return out


def _finish(batch, steps):
    res = []
    for lat, eng in zip(batch.lattices, batch.engines):
        eng.cur = batch.parity
        _finalize_state(lat, eng, steps)
        res.append((lat.g.copy(), eng.drag_rows(steps - 5, steps)))
    return res


# persistent: 1 work-queue kernels, 0 one block per tile; rounds: block-widths
# of vector groups per bulk tile; tma: the TMA-staged bulk kernel (16-bit
# forms; 1 the form's shape, 2 half its warps per block; the single lattices
# step through the TMA-staged kernel too, so this also compares the two bulk
# kernels where tma is 0); groups: lattices split into that many batches
# advanced concurrently on their own streams.
@pytest.mark.parametrize("precision,persistent,vec_bytes,rounds,tma,groups", [
    ("f16s", 1, 16, 1, 0, 1), ("f64", 1, 16, 1, 0, 1), ("f16sr", 0, 8, 1, 0, 1),
    ("f16sr", 1, 8, 4, 0, 1), ("f16sr", 0, 16, 3, 0, 1), ("q60", 0, 16, 1, 0, 1),
    ("f16s", 1, 16, 1, 1, 1), ("f16sr", 0, 16, 1, 1, 1), ("bf16s", 0, 16, 1, 1, 1),
    ("bf16sr", 1, 16, 1, 1, 1), ("f16sr", 0, 16, 1, 1, 2), ("q60", 0, 16, 1, 0, 3),
    ("f16s", 0, 16, 1, 2, 2), ("bf16sr", 1, 16, 1, 2, 1)])
def test_batch_equals_single_lattices(cuda, precision, persistent, vec_bytes, rounds, tma,
                                      groups):
    steps = 120
    cfg = default_config()
    cfg.update(persistent=persistent, vec_bytes=vec_bytes, bulk_threads=64, tile_rounds=rounds,
               bulk_tma=tma, streams=groups)
    b = Batch(_apps(), precision=precision, config=cfg)
    b.advance(steps, k=40)
    b.check()
    got = _finish(b, steps)
    info = b.info()
    b.close()
    assert info["lattices"] == 5 and info["drag_items"] == 3 and info["groups"] == groups

    s = Batch(_apps(), precision=precision)
    for eng in s.engines:
        eng.steps(1, steps, graph=True)
    ref = _finish(type("B", (), {"lattices": s.lattices, "engines": s.engines,
                                 "parity": s.engines[0].cur})(), steps)
    s.close()
    for (g1, d1), (g2, d2) in zip(got, ref):
        assert np.array_equal(g1, g2)
        assert np.array_equal(d1, d2)


def test_sweep_generator_is_seeded_and_in_range():
    a = sweep_apps(seed=7, n_cavity=6, n_channel=6)
    b = sweep_apps(seed=7, n_cavity=6, n_channel=6)
    assert [x.nx for x in a] == [x.nx for x in b]
    for x in a[:6]:
        assert 64 <= x.ny <= 512 and 100.0 <= x.Re_lbm <= 1000.0 and x.nx == x.ny
    for x in a[6:]:
        assert 64 <= x.ny <= 256 and x.nx == 4 * x.ny and 1 <= len(x.obstacles) <= 6
        assert 100.0 <= x.Re_lbm <= 2000.0
        assert x.tau_lbm >= 0.53 - 1e-12


def test_autotune_puts_the_lattices_back(cuda):
    """The autotuner's trials advance the lattices; afterwards every lattice
    holds the state it had before them, and the batch continues from the
    same iteration (a tiny candidate space keeps this short)."""
    import torch
    from lbm_gb300.batch import autotune
    b = Batch(_apps(), precision="f16sr")
    b.advance(20, k=10)
    torch.cuda.synchronize()
    before = [e.f[e.cur].clone() for e in b.engines]
    it0, parity0 = b.it, b.parity
    space = {"persistent": [0], "tile_rounds": [1], "vec_bytes": [16], "bulk_threads": [64],
             "k_steps": [10]}
    best, trials = autotune(b, steps=20, space=space, k_space=(10,), stream_space=(2,))
    assert b.it == it0 and b.parity == parity0
    for e, f in zip(b.engines, before):
        assert e.cur == parity0
        assert torch.equal(e.f[e.cur], f)
    assert len(trials) >= 3 and best["k_steps"] == 10
    b.advance(10, k=10)
    b.check()
    b.close()
