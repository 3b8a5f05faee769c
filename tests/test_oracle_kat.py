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
    """Philox4x32-10 known-answer vectors published with Random123 (Salmon et al. 2011)."""
    import ctypes as C
    L = oracle_mod.lib()
    out = (C.c_uint32 * 4)()
    # counter (c0,c1,c2,c3) = (step_lo, step_hi, a, b); key = (seed_lo, seed_hi)
    L.orc_philox(0, 0, 0, 0, out)
    assert list(out) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    L.orc_philox(0xFFFFFFFFFFFFFFFF, -1, 0xFFFFFFFF, 0xFFFFFFFF, out)
    assert list(out) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    step = ((0x85A308D3 << 32) | 0x243F6A88) - (1 << 64)  # as a signed 64-bit counter
    L.orc_philox(0x299F31D0A4093822, step, 0x13198A2E, 0x03707344, out)
    assert list(out) == [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


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
