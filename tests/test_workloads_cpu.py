"""The synthetic-workload generators: the whole-array layered generator has the
law of the per-layer one (predecessor counts, pools, distinct predecessors,
uniform pool positions), and serving requests have the configured sizes."""
from __future__ import annotations

import numpy as np

from mc_dagprop_gb300 import workloads as W


def _check_structure(flat, width, back, max_preds=4):
    off, src, tgt = flat["pred_offsets"], flat["pred_src"], flat["target"]
    cnt = np.diff(off)
    assert (cnt >= 1).all() and (cnt <= max_preds).all()
    for k, t in enumerate(tgt):
        s = src[off[k]:off[k + 1]]
        layer = t // width
        assert len(set(s.tolist())) == len(s)
        assert ((s // width < layer) & (s // width >= max(0, layer - back))).all()
    assert np.array_equal(flat["act_dst"], np.repeat(tgt, cnt))
    assert len(flat["act_idx"]) == len(src)


def test_fast_layered_dag_law():
    rng = np.random.default_rng(5)
    fast = W.layered_dag_fast(rng, 400, 20, 3, [1, 2], 1800.0)
    slow = W.layered_dag(5, 400, 20, 3, [1, 2], 1800.0)
    for f in (fast, slow):
        _check_structure(f, 20, 3)
    cf, cs = np.diff(fast["pred_offsets"]), np.diff(slow["pred_offsets"])
    assert abs(cf.mean() - cs.mean()) < 0.05 and abs(cf.mean() - 2.5) < 0.05
    # pool positions of full-pool events are uniform (60 positions, ~7,400 picks)
    off = fast["pred_offsets"]
    pos = np.concatenate([fast["pred_src"][off[k]:off[k + 1]] - (t // 20 - 3) * 20
                          for k, t in enumerate(fast["target"]) if t >= 60])
    h = np.bincount(pos, minlength=60)
    chi2 = ((h - h.mean()) ** 2 / h.mean()).sum()
    assert chi2 < 100.0, chi2  # 59 degrees of freedom: p ~ 1e-3 at 95
    # the first-listed predecessor is not biased toward either end of the pool
    first = np.array([fast["pred_src"][off[k]] - (t // 20 - 3) * 20 for k, t in enumerate(fast["target"])
                      if t >= 60 and off[k + 1] - off[k] >= 2])
    assert abs(first.mean() - 29.5) < 1.5


def test_fresh_requests_sizes():
    rng = np.random.default_rng(9)
    reqs = [W.fresh_request(rng) for _ in range(300)]
    ev = np.array([len(r[0]["earliest"]) for r in reqs])
    ns = np.array([r[2] for r in reqs])
    assert ev.min() >= 100 and ev.max() <= 21_000
    assert ns.min() >= 4096 and ns.max() <= 65_536
    # log-uniform over [200, 20000]: the mean of log(events / 200) is log(100) / 2 = 2.30
    assert abs(np.log(ev / 200).mean() - np.log(100) / 2) < 0.3
    assert len({r[3] for r in reqs}) == 300
