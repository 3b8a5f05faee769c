"""Cluster-pair occupancy of the pair workloads: a measured property of the configurations behind
the choice of a per-particle Verlet list over a cluster-pair kernel (Pall & Hess, Comput. Phys.
Commun. 184 (2013) 2641: i-clusters of M particles against j-clusters of M, a warp per cluster
pair, every M x M slot tested, j forces reduced in the warp and added once per j particle).

Clusters are built the way that scheme builds them: columns on an x-y grid of width (M/rho)^(1/3),
particles of a column sorted by z and cut into runs of M.  A cluster pair is listed when the gap
between the two bounding boxes is below the list range rc + skin.  On states 200 oracle steps
from the lattice start, the tests measure

* occupancy: interacting pairs (r < rc) / M x M slots of the listed cluster pairs;
* j atomics per interacting pair: (cluster pair, j particle) combinations with at least one
  interaction, per interacting pair (one atomic add of a j force per combination);
* list entries per interacting pair of the full per-particle list that the library builds.

Printed with -s; the asserts pin the regime the design relies on: at the WCA cut-off a 4 x 4
cluster pair holds well under one interacting pair, so a warp of such pairs would run the pair
arithmetic (the Philox draw, Box-Muller, LJ, DPD) for a few lanes, and the j-force atomics stay
near one per pair, the count that made evaluating each pair once slower than the full list."""
import os

import numpy as np
from scipy.spatial import cKDTree

from mfa_brush_gb300 import configs

RC_WCA = 2.0 ** (1.0 / 6.0)
SKIN = 0.5


def _clusters(r, L, M):
    """Cluster id of every particle: x-y columns of width (M / rho)^(1/3), z-sorted runs of M."""
    n = len(r)
    rho = n / (L[0] * L[1] * (r[:, 2].max() - r[:, 2].min()))
    nc = max(1, int(round(L[0] / (M / rho) ** (1.0 / 3.0))))
    ix = np.minimum(((r[:, 0] % L[0]) / (L[0] / nc)).astype(int), nc - 1)
    iy = np.minimum(((r[:, 1] % L[1]) / (L[1] / nc)).astype(int), nc - 1)
    col = ix * nc + iy
    order = np.lexsort((r[:, 2], col))
    sizes = np.bincount(col, minlength=nc * nc)
    starts = np.r_[0, np.cumsum(sizes)[:-1]]
    pos = np.arange(n) - np.repeat(starts, sizes)
    per_col = (sizes + M - 1) // M
    base = np.r_[0, np.cumsum(per_col)[:-1]]
    cid = np.empty(n, np.int64)
    cid[order] = np.repeat(base, sizes) + pos // M
    return cid, int(per_col.sum())


def cluster_pair_stats(r, L, M, rc, skin=SKIN):
    cid, ncl = _clusters(r, L, M)
    box = [L[0], L[1], 1e9]
    xw = np.column_stack([r[:, 0] % L[0], r[:, 1] % L[1], r[:, 2]])
    tree = cKDTree(xw, boxsize=box)
    inter = tree.query_pairs(rc, output_type="ndarray")
    listed = tree.query_pairs(rc + skin, output_type="ndarray")
    order = np.argsort(cid, kind="stable")
    cnt = np.bincount(cid, minlength=ncl)
    bounds = np.r_[0, np.cumsum(cnt)]
    lo, hi = np.zeros((ncl, 3)), np.zeros((ncl, 3))
    for k in range(ncl):
        p = r[order[bounds[k]:bounds[k + 1]]].copy()
        p[:, :2] -= L[:2] * np.round((p[:, :2] - p[0, :2]) / L[:2])  # a column never spans the box
        lo[k], hi[k] = p.min(0), p.max(0)
    cen, half = (lo + hi) / 2, (hi - lo) / 2
    ct = cKDTree(np.column_stack([cen[:, 0] % L[0], cen[:, 1] % L[1], cen[:, 2]]), boxsize=box)
    cand = ct.query_pairs(rc + skin + 2 * np.sqrt((half ** 2).sum(1)).max(), output_type="ndarray")
    d = cen[cand[:, 1]] - cen[cand[:, 0]]
    d[:, :2] -= L[:2] * np.round(d[:, :2] / L[:2])
    gap = np.maximum(np.abs(d) - half[cand[:, 0]] - half[cand[:, 1]], 0.0)
    cp = cand[(gap ** 2).sum(1) < (rc + skin) ** 2]
    slots = int((cnt[cp[:, 0]] * cnt[cp[:, 1]]).sum() + (cnt * (cnt - 1) // 2).sum())
    ci, cj = cid[inter[:, 0]], cid[inter[:, 1]]
    lo_c, hi_c = np.minimum(ci, cj), np.maximum(ci, cj)
    jpart = np.where(ci <= cj, inter[:, 1], inter[:, 0])
    combos = len(np.unique(np.stack([lo_c, hi_c, jpart], 1), axis=0))
    n_int = len(inter)
    return {"M": M, "cluster_pairs": len(cp) + ncl, "slots": slots, "interacting": n_int,
            "occupancy": n_int / slots, "j_atomics_per_pair": combos / n_int,
            "list_entries_per_pair": len(listed) / n_int}


def _relaxed(oracle_mod, p, system):
    s, a_type, r0, v = system
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    o.step(200, min(8, os.cpu_count() or 1), 0)
    r = o.state()[0]
    o.close()
    assert np.all(np.isfinite(r))
    return r, np.array(list(s.boundary))


def test_cluster_pairs_at_the_wca_cut_off(oracle_mod):
    """Replica 0 of the 256-replica workload (18,883 particles, WCA + FENE + DPD)."""
    p = configs.wca_params(gamma=5.0, kT=1.0, dt=0.005)
    (sysm,) = configs.replicas(256, 2024, indices=[0])
    r, L = _relaxed(oracle_mod, p, sysm)
    for M in (4, 8):
        st = cluster_pair_stats(r, L, M, RC_WCA)
        print("WCA", {k: round(v, 3) if isinstance(v, float) else v for k, v in st.items()})
        assert st["occupancy"] < 0.08
        assert st["j_atomics_per_pair"] > 0.6
        assert 2.5 < st["list_entries_per_pair"] < 3.8


def test_cluster_pairs_in_a_melt(oracle_mod):
    """A 20 x 20 x 40 melt-in-brush channel (13,600 particles); every pair counted at the melt's
    2 x 2^(1/6) cut-off (brush-brush pairs are WCA in the model, so the occupancy is an upper
    bound)."""
    p, sysm = configs.melt_brush(L=20.0, D=40.0)
    r, L = _relaxed(oracle_mod, p, sysm)
    for M in (4, 8):
        st = cluster_pair_stats(r, L, M, 2.0 * RC_WCA)
        print("melt", {k: round(v, 3) if isinstance(v, float) else v for k, v in st.items()})
        assert st["occupancy"] < 0.25
        assert st["list_entries_per_pair"] < 2.5


def test_cluster_pairs_in_two_liquids(oracle_mod):
    """A 20 x 20 x 16 two-liquid channel (brushes, liquids A and B layered, 5,120 particles); every
    pair counted at the liquids' 2 x 2^(1/6) cut-off (an upper bound, as for the melt)."""
    from mfa_brush_gb300 import md
    p, _ = md.derive(configs.two_liquid_inputs(f_x=0.01))
    sysm = configs.two_liquid_channel(L=20.0, D=16.0, seed=5)
    r, L = _relaxed(oracle_mod, p, sysm)
    for M in (4, 8):
        st = cluster_pair_stats(r, L, M, 2.0 * RC_WCA)
        print("two liquids", {k: round(v, 3) if isinstance(v, float) else v for k, v in st.items()})
        assert st["occupancy"] < 0.25
        assert st["list_entries_per_pair"] < 2.5
