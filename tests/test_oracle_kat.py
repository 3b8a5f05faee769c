"""The oracle against the reference's own known-answer values (tests/golden/try/kat.json, taken from
the reference's try/ run: try/log and try/mfa_output) and the product's host-side table derivation
against the oracle's.  CPU only."""
import json
import os

import numpy as np

from conftest import GOLDEN


def kat():
    with open(os.path.join(GOLDEN, "try", "kat.json")) as f:
        return json.load(f)


def test_tables_match_log(try_deck, oracle_mod):
    inp, p, s, *_ = try_deck
    po, so = oracle_mod.derive_params(inp)
    K = kat()
    # init_params.f90:742-745 print sqrt(range_2(:,i)) per particle i, f10.5
    np.testing.assert_allclose(np.sqrt(po.table("range_2")).T, np.array(K["cutoffs"]), atol=5e-6)
    # init_params.f90:758-761 print 4*e_shift(:,i), f10.5
    np.testing.assert_allclose(4 * po.table("e_shift").T, np.array(K["shifts"]), atol=5e-6)
    assert abs(po.r_cut_max - K["r_cut_max"]) < 5e-6
    assert abs(np.sqrt(po.r_cut_dpd_2) - K["r_cut_dpd"]) < 5e-6
    # 0.4 as a default-REAL literal, printed list-directed with 15 digits: 0.400000005960464
    assert abs(po.skin - K["skin"]) < 1e-15 and po.skin != 0.4


def test_product_tables_equal_oracle(try_deck, oracle_mod):
    inp, p, s, *_ = try_deck
    po, so = oracle_mod.derive_params(inp)
    for name in ("range_2", "inv_range_2", "e_shift", "epsil", "sigma", "sigma_2"):
        assert np.array_equal(p.table(name), po.table(name)), name
    for f in ("r_cut_max", "r_cut_dpd_2", "sig", "friction1", "k_chain", "r_chain_2", "k_bend", "k_or", "skin", "dt"):
        assert getattr(p, f) == getattr(po, f), f
    assert list(s.boundary) == list(so.boundary) == [30.0, 20.0, 40.0]
    assert (s.n_mon_tot, s.n_part, s.s_time) == (so.n_mon_tot, so.n_part, so.s_time) == (6000, 6000, 2)


def test_first_lj_energy(try_deck, oracle_mod):
    """check_fluid_fluid (util.f90:284-330) of try/conf_old printed -1131.60193205932."""
    inp, p, s, a_type, r0, v, a = try_deck
    o = oracle_mod.Oracle(p, s, a_type, r0, v, a)
    e2 = o.check_fluid_fluid()
    assert abs(e2 - kat()["v_fluid_fluid_check"]) < 1e-10
    o.fluid_fluid()  # linked-cell traversal (fluid_fluid.f90:71-477) gives the same total
    assert abs(o.energies()["v_fluid_fluid"] - e2) < 1e-10 * abs(e2)


def test_first_vcm(try_deck):
    """init_config.f90:336-343: first centre-of-mass velocity of try/conf_old."""
    inp, p, s, a_type, r0, v, a = try_deck
    m = np.array([p.mass_type[t - 1] for t in a_type])
    vcm = (m[:, None] * v).sum(0) / m.sum()
    np.testing.assert_allclose(vcm, kat()["first_vcm"], atol=5e-6)


def test_binning_boxes(try_deck):
    """try/mfa_output: the BIN_TYPE 0 grid int(L/(r_cut_max+skin)) = 11 7 15, sizes L/n."""
    inp, p, s, *_ = try_deck
    n = [int(L / (p.r_cut_max + p.skin)) for L in s.boundary]
    assert n == kat()["binning_boxes"]
    np.testing.assert_allclose([L / k for L, k in zip(s.boundary, n)], kat()["binning_distances"], atol=5e-7)


def test_philox_known_answers(oracle_mod):
    """Philox2x32-10 known-answer vectors published with Random123 (Salmon et al. 2011):
    counter (c0, c1), key k."""
    import ctypes as C
    L = oracle_mod.lib()
    out = (C.c_uint32 * 2)()
    L.orc_philox2x32(0, 0, 0, out)
    assert list(out) == [0xFF1DAE59, 0x6CD10DF2]
    L.orc_philox2x32(0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, out)
    assert list(out) == [0x2C3F628B, 0xAB4FD7AD]


def _philox2x32_np(c0, c1, k):
    """Vectorised Philox2x32-10 (the published round function), for large-sample checks."""
    M, W, m32 = np.uint64(0xD256D193), np.uint64(0x9E3779B9), np.uint64(0xFFFFFFFF)
    c0, c1, k = c0.astype(np.uint64), c1.astype(np.uint64), np.uint64(k)
    for r in range(10):
        if r:
            k = (k + W) & m32
        p = M * c0
        c0, c1 = (p >> np.uint64(32)) ^ k ^ c1, p & m32
    return c0, c1


def test_pair_noise_large_sample(oracle_mod):
    """The pair noise over 10^6 draws for three counter patterns (neighbouring tags, a stride, a
    block) and two keys: mean and variance of g within 5 standard errors, every used bit of both
    words set half the time; the vectorised restatement equals orc_pair_gauss draw for draw."""
    L = oracle_mod.lib()
    n = 1_000_000
    i = np.arange(n, dtype=np.uint64)
    for seed, step in ((2024, 7), (0x9E3779B97F4A7C15, 123456)):
        k = L.orc_pair_key(seed, step)
        for a, b in ((i, i + 1), (i, i + 7), (i % 1000, i // 1000 + 1000)):
            c0, c1 = _philox2x32_np(a, b, k)
            u1 = ((c0 >> np.uint64(9)).astype(np.float64) + 0.5) / 8388608.0
            u2 = (c1 >> np.uint64(9)).astype(np.float64) / 8388608.0
            g = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
            for t in (0, 17, n - 1):
                assert g[t] == oracle_mod.pair_gauss(seed, step, int(a[t]), int(b[t]))
            assert abs(g.mean()) < 5.0 / np.sqrt(n)
            assert abs(g.var() - 1.0) < 5.0 * np.sqrt(2.0 / n)
            for w in (c0, c1):
                f = np.array([((w >> np.uint64(j)) & np.uint64(1)).mean() for j in range(9, 32)])
                assert np.abs(f - 0.5).max() < 5.0 * 0.5 / np.sqrt(n)


def test_pair_key_distinct_over_steps(oracle_mod):
    """A replica's noise keys of distinct steps differ (the step enters by XOR), and replicas with
    consecutive seeds get unrelated keys (the seed is hashed)."""
    L = oracle_mod.lib()
    ks = [L.orc_pair_key(12345, t) for t in range(5000)]
    assert len(set(ks)) == 5000
    k0 = [L.orc_pair_key(s, 0) for s in range(64)]
    assert len(set(k >> 24 for k in k0)) > 32


def test_pair_gauss_is_symmetric_and_normal(oracle_mod):
    g = np.array([oracle_mod.pair_gauss(7, 11, i, i + 1 + (i % 13)) for i in range(20000)])
    assert oracle_mod.pair_gauss(7, 11, 3, 9) == oracle_mod.pair_gauss(7, 11, 9, 3)
    assert abs(g.mean()) < 0.03 and abs(g.std() - 1) < 0.03


def test_product_tables_equal_oracle_explicit_walls(oracle_mod):
    """WALL 1 + DPD_CUT_OFF: the product's table derivation equals the oracle's."""
    from mfa_brush_gb300 import configs, md
    inp = configs.wca_inputs(gamma=5.0, wall=1, dpd_cut_off=1.0)
    p, _ = md.derive(inp)
    po, _ = oracle_mod.derive_params(inp)
    assert p.n_type == po.n_type == 4
    for name in ("range_2", "inv_range_2", "e_shift", "epsil", "sigma", "sigma_2"):
        assert np.array_equal(p.table(name), po.table(name)), name
    for f in ("r_cut_max", "r_cut_dpd_2", "sig", "friction1", "skin"):
        assert getattr(p, f) == getattr(po, f), f
