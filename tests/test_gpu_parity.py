"""GPU parity: the CUDA path (through the C ABI) against the oracle on the same inputs.

Tolerances: FP64 path -- forces 1e-9 relative to max(|F_i|, 1e-3 F_rms), energies 1e-10;
mixed path -- forces: max_i |dF_i| / F_rms <= 1e-5 and the 99th percentile of the per-particle
relative error <= 1e-5 (conftest.mixed_force_err); energies 1e-5 relative.  Cell assignment,
half-shell tables and interacting-pair sets are compared exactly."""
import numpy as np
import pytest

from conftest import assert_force_parity, rel_force_err
from mfa_brush_gb300 import abi, configs, md

pytestmark = pytest.mark.gpu

TOL_E = {"fp64": 1e-10, "mixed": 1e-5}


def gpu_and_oracle(oracle_mod, p, s, a_type, r0, v, a, precision):
    g = md.MdSystem(p, s, a_type, r0, v, a, precision=precision)
    o = oracle_mod.Oracle(p, s, a_type, r0, v, a)
    return g, o


def rel(x, y):
    return abs(x - y) / max(abs(y), 1e-300)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_try_fluid_fluid(gpu, try_deck, oracle_mod, precision):
    """LJ + DPD (own cut-off, Philox noise) on try/conf_old."""
    inp, p, s, a_type, r0, v, a = try_deck
    g, o = gpu_and_oracle(oracle_mod, p, s, a_type, r0, v, a, precision)
    g.zero_force()
    vff, _ = g.fluid_fluid()
    f = g.state()[3]
    o.zero_force()
    o.fluid_fluid()
    fo = o.state()[3]
    assert rel(vff[0], o.energies()["v_fluid_fluid"]) < TOL_E[precision]
    assert rel(vff[0], -1131.60193205932) < max(TOL_E[precision], 1e-12)
    assert_force_parity(f, fo, precision)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("routine,key", [("intra_molec", "v_intra_molec"), ("bending", "v_bend"),
                                         ("orientation", "v_or"), ("fluid_wall", "v_fluid_wall")])
def test_try_single_routines(gpu, try_deck, oracle_mod, precision, routine, key):
    inp, p, s, a_type, r0, v, a = try_deck
    g, o = gpu_and_oracle(oracle_mod, p, s, a_type, r0, v, a, precision)
    g.zero_force()
    e = getattr(g, routine)()
    o.zero_force()
    getattr(o, routine)()
    tol_e = 1e-10 if (routine == "fluid_wall" or precision == "fp64") else TOL_E[precision]
    assert rel(e[0], o.energies()[key]) < tol_e
    assert_force_parity(g.state()[3], o.state()[3], "fp64" if routine == "fluid_wall" else precision)


def test_try_md_steps_fp64(gpu, try_deck, oracle_mod):
    """Five md_main iterations through the per-routine drop-ins vs the oracle."""
    inp, p, s, a_type, r0, v, a = try_deck
    g, o = gpu_and_oracle(oracle_mod, p, s, a_type, r0, v, a, "fp64")
    for _ in range(5):
        eg = g.md_step()[0]
    o.step(5, 1, 0)
    r, vv, aa, f = g.state()
    ro, vo, ao, fo = o.state()
    d = r - ro
    d[:, :2] -= np.array(list(s.boundary))[:2] * np.round(d[:, :2] / np.array(list(s.boundary))[:2])
    assert np.abs(d).max() < 1e-9
    assert np.abs(vv - vo).max() < 1e-7 * max(1.0, np.abs(vo).max())
    eo = o.energies()
    for k in ("v_fluid_fluid", "v_intra_molec", "v_bend", "v_or", "v_fluid_wall", "t_fluid"):
        assert rel(eg[k], eo[k]) < 1e-8, k


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_explicit_walls_fluid_fluid(gpu, oracle_mod, precision):
    """WALL 1 (explicit wall beads on a 1 sigma lattice, DPD with its own 1 sigma cut-off): pair
    forces on the mobile particles and the LJ energy, wall-wall pairs included."""
    p = configs.wca_params(gamma=5.0, wall=1, dpd_cut_off=1.0)
    s, a_type, r0, v = configs.explicit_wall_channel(seed=3)
    g, o = gpu_and_oracle(oracle_mod, p, s, a_type, r0, v, None, precision)
    g.zero_force()
    vff, _ = g.fluid_fluid()
    o.zero_force()
    o.fluid_fluid()
    m = s.n_mon_tot
    assert rel(vff[0], o.energies()["v_fluid_fluid"]) < TOL_E[precision]
    assert_force_parity(g.state()[3][:m], o.state()[3][:m], precision)


def test_explicit_walls_md_steps_fp64(gpu, oracle_mod):
    """Five md_main iterations with explicit walls through the drop-ins vs the oracle."""
    p = configs.wca_params(gamma=5.0, wall=1, dpd_cut_off=1.0)
    s, a_type, r0, v = configs.explicit_wall_channel(seed=4)
    g, o = gpu_and_oracle(oracle_mod, p, s, a_type, r0, v, None, "fp64")
    for _ in range(5):
        eg = g.md_step()[0]
    o.step(5, 1, 0)
    r, vv, aa, f = g.state()
    ro, vo, ao, fo = o.state()
    L = np.array(list(s.boundary))
    d = r - ro
    d[:, :2] -= L[:2] * np.round(d[:, :2] / L[:2])
    assert np.abs(d).max() < 1e-9
    assert np.abs(vv - vo).max() < 1e-7 * max(1.0, np.abs(vo).max())
    eo = o.energies()
    for k in ("v_fluid_fluid", "v_intra_molec", "t_fluid"):
        assert rel(eg[k], eo[k]) < 1e-8, k


def test_fused_step_matches_drop_ins(gpu, try_deck):
    """mfa_step(n) (graph-captured, fused integrator) reproduces n per-routine md_main steps."""
    inp, p, s, a_type, r0, v, a = try_deck
    g1 = md.MdSystem(p, s, a_type, r0, v, a, precision="fp64")
    g2 = md.MdSystem(p, s, a_type, r0, v, a, precision="fp64")
    for _ in range(7):
        e1 = g1.md_step()[0]
    g2.step(7)
    e2 = g2.energies()[0]
    s1, s2 = g1.state(), g2.state()
    assert np.abs(s1[0] - s2[0]).max() < 1e-10
    assert np.abs(s1[1] - s2[1]).max() < 1e-8
    for k in ("v_fluid_fluid", "v_intra_molec", "v_bend", "v_or", "v_fluid_wall", "t_fluid", "e_total"):
        assert rel(e1[k], e2[k]) < 1e-9, k
    assert g2.step_index() == s.s_time + 7


def test_try_steps_mixed(gpu, try_deck, oracle_mod):
    """Ten fused mixed-precision steps against ten FP64 oracle steps (dt = 2e-4): positions within
    1e-8 sigma, velocities within 1e-5 relative to their RMS, energies within 1e-5."""
    inp, p, s, a_type, r0, v, a = try_deck
    g, o = gpu_and_oracle(oracle_mod, p, s, a_type, r0, v, a, "mixed")
    g.step(10)
    o.step(10, 1, 0)
    r, vv, aa, f = g.state()
    ro, vo, ao, fo = o.state()
    L = np.array(list(s.boundary))
    d = r - ro
    d[:, :2] -= L[:2] * np.round(d[:, :2] / L[:2])
    assert np.abs(d).max() < 1e-8
    assert np.abs(vv - vo).max() < 1e-5 * np.sqrt(np.mean(vo ** 2))
    eg, eo = g.energies()[0], o.energies()
    for k in ("v_fluid_fluid", "v_intra_molec", "v_bend", "v_or", "v_fluid_wall", "t_fluid"):
        assert rel(eg[k], eo[k]) < 1e-5, k


@pytest.mark.parametrize("l_box", [1, 2])
def test_reference_cell_list_bit_exact(gpu, try_deck, oracle_mod, l_box):
    """get_cell on the reference's own grid (make_binning with r_cut_max): identical cells."""
    inp, p, s, a_type, r0, v, a = try_deck
    g, o = gpu_and_oracle(oracle_mod, p, s, a_type, r0, v, a, "fp64")
    o.make_cell_list(l_box)
    cg, ng, ncg = g.cell_list(0, l_box)
    co, no, nco = o.cell_info()
    assert list(ncg) == list(nco)
    assert np.array_equal(cg, co)
    assert np.array_equal(ng, no)


@pytest.mark.parametrize("n_cells,n_nei", [((11, 7, 15), 13), ((13, 8, 17), 13), ((26, 17, 35), 62)])
def test_half_shell_table_bit_exact(gpu, oracle_mod, n_cells, n_nei):
    assert np.array_equal(md.cell_neigh_list(n_cells, n_nei), oracle_mod.cell_neigh_list(n_cells, n_nei))


def test_interacting_pairs_identical(gpu, try_deck, oracle_mod):
    inp, p, s, a_type, r0, v, a = try_deck
    g, o = gpu_and_oracle(oracle_mod, p, s, a_type, r0, v, a, "fp64")
    pg = g.pair_list(0)
    po = o.pair_list()
    sg = set(map(tuple, np.sort(pg, axis=1).tolist()))
    so = set(map(tuple, po.tolist()))
    assert len(pg) == len(sg) and sg == so


def test_wca_channel_fused_mixed_vs_oracle(gpu, oracle_mod):
    """The bench model (WCA + FENE + DPD, single cut-off, so the list builder and the pair
    screening take their uniform-cut-off form, and the bonded terms run inside the pair kernel):
    10 fused mixed steps against 10 FP64 oracle steps with the same noise."""
    p = configs.wca_params(gamma=5.0)
    s, a_type, r0, v = configs.brush_channel(16.0, 14.0, 0.2, 25, seed=21)
    g, o = gpu_and_oracle(oracle_mod, p, s, a_type, r0, v, None, "mixed")
    g.step(10)
    o.step(10, 1, 0)
    r, vv, aa, f = g.state()
    ro, vo, ao, fo = o.state()
    L = np.array(list(s.boundary))
    d = r - ro
    d[:, :2] -= L[:2] * np.round(d[:, :2] / L[:2])
    assert np.abs(d).max() < 1e-7
    assert np.abs(vv - vo).max() < 1e-4 * np.sqrt(np.mean(vo ** 2))
    eg, eo = g.energies()[0], o.energies()
    for k in ("v_fluid_fluid", "v_intra_molec", "v_fluid_wall", "t_fluid"):
        assert rel(eg[k], eo[k]) < 1e-5, k


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_replicas_equal_single(gpu, precision):
    """A replica inside a batch gets a bit-identical trajectory to the same replica run alone,
    rebuilds included: each replica is rebuilt when its own particles have moved half the skin
    (check_skin.f90 decides per system), so its sort order and lists do not depend on the others.
    The cold replica (solvent on a lattice of spacing > 2^(1/6), so no potential energy to
    release, velocities scaled by 0.1) is rebuilt less often than the others."""
    p = configs.wca_params(gamma=5.0)
    reps = [configs.brush_channel(15.0, 12.0, 0.2, 20, seed=11),
            configs.brush_channel(18.0, 15.0, 0.1, 35, seed=12),
            configs.brush_channel(16.0, 10.0, 0.0, 10, rho=0.35, a_max=1.25, seed=13)]
    s2, a2, r2, v2 = reps[2]
    reps[2] = (s2, a2, r2, v2 * 0.1)
    systems, a_type, r0, v = configs.concat(reps)
    # an ample list capacity: a capacity growth rebuilds every replica at once
    gb = md.MdSystem(p, systems, a_type, r0, v, precision=precision, nbr_capacity=160)
    gb.step(60)
    rb, vb, ab, fb = gb.state()
    counts = gb.replica_rebuild_counts()
    assert counts.min() >= 0 and counts.max() >= 2 and counts[2] < counts.max()
    off = 0
    for k, (s, at, r, vv) in enumerate(reps):
        g1 = md.MdSystem(p, s, at, r, vv, precision=precision, nbr_capacity=160)
        g1.step(60)
        r1, v1, a1, f1 = g1.state()
        assert g1.replica_rebuild_counts()[0] == counts[k]
        n = s.n_part
        assert np.array_equal(r1, rb[off:off + n])
        assert np.array_equal(v1, vb[off:off + n])
        off += n


def test_profiles_match_oracle(gpu, oracle_mod):
    p = configs.wca_params(gamma=5.0)
    p.flags.profiles = 1
    s, a_type, r0, v = configs.small_channel()
    g = md.MdSystem(p, s, a_type, r0, v, precision="fp64")
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    for _ in range(6):
        g.md_step(profiles=True)
    o.step(6, 1, 1)
    dg, vg, v2g, ng = g.profiles(0)
    do, vo, v2o, no = o.profiles()
    assert ng == no == 6
    assert np.array_equal(dg, do)
    assert np.abs(vg - vo).max() < 1e-9 and np.abs(v2g - v2o).max() < 1e-9


def charged_system(n_kmax=5):
    inp = configs.wca_inputs(gamma=1.0, thermostat=0)
    inp.flags.system = 3
    inp.charge[1] = -1.0  # brush beads
    inp.charge[2] = 1.0   # solvent
    inp.alpha_c = 0.81
    inp.n_kmax = n_kmax
    inp.rc_coul = 3.0
    p, _ = md.derive(inp)
    s, a_type, r0, v = configs.brush_channel(10.0, 10.0, 0.08, 10, rho=0.5, seed=21)
    return p, s, a_type, r0, v


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ewald_matches_oracle(gpu, oracle_mod, precision):
    p, s, a_type, r0, v = charged_system()
    g, o = gpu_and_oracle(oracle_mod, p, s, a_type, r0, v, None, precision)
    o.ewald_init()
    # real space (inside fluid_fluid)
    g.zero_force(); _, vc = g.fluid_fluid(); f_real = g.state()[3]
    o.zero_force(); o.fluid_fluid(); fo_real = o.state()[3]; vco = o.energies()["v_coul"]
    assert rel(vc[0], vco) < TOL_E[precision]
    assert_force_parity(f_real, fo_real, precision)
    # k space
    g.zero_force(); uk = g.ewald_k()[0]; fk = g.state()[3]
    o.zero_force(); uko = o.ewald_k(); fko = o.state()[3]
    assert rel(uk, uko) < (1e-10 if precision == "fp64" else 1e-5)
    assert_force_parity(fk, fko, precision)
    # slab dipole correction
    g.zero_force(); ud = g.dipolar_correction()[0]; fd = g.state()[3]
    o.zero_force(); udo = o.dipolar_correction(); fdo = o.state()[3]
    assert rel(ud, udo) < 1e-10
    assert np.abs(fd - fdo).max() < 1e-10 * max(1.0, np.abs(fdo).max())


def test_deterministic_and_momentum(gpu):
    """Two identical runs are bit-identical; pair forces conserve momentum (noise is antisymmetric)."""
    p = configs.wca_params(gamma=5.0)
    reps = configs.replicas(6, seed=5)
    systems, a_type, r0, v = configs.concat(reps)
    out = []
    for _ in range(2):
        g = md.MdSystem(p, systems, a_type, r0, v, precision="mixed")
        g.step(40)
        out.append(g.state())
    for x, y in zip(out[0], out[1]):
        assert np.array_equal(x, y)
    g.zero_force()
    g.fluid_fluid()
    f = g.state()[3]
    assert np.abs(f.sum(0)).max() < 1e-5 * np.abs(f).sum()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ewald_wide_kset_matches_oracle(gpu, oracle_mod, precision):
    """n_kmax = 17: nx runs over -17..17, so the structure factor takes two 32-slot groups of
    k_ks_rho and the mixed force takes the one-k-at-a-time kernel instead of the register-resident
    slot table (which holds nxm <= 15)."""
    p, s, a_type, r0, v = charged_system(n_kmax=17)
    g, o = gpu_and_oracle(oracle_mod, p, s, a_type, r0, v, None, precision)
    nk, nq = g.kspace_info()
    assert nk == len(o.kvecs()) and nk > 20000 and nq > 0  # kvecs() also sets the oracle's sum up
    g.zero_force(); uk = g.ewald_k()[0]; fk = g.state()[3]
    o.zero_force(); uko = o.ewald_k(); fko = o.state()[3]
    assert rel(uk, uko) < (1e-10 if precision == "fp64" else 1e-5)
    assert_force_parity(fk, fko, precision)


def test_ewald_very_wide_kset_fp64_smaller_force_chunks(gpu, oracle_mod):
    """n_kmax = 40 in FP64: the one-k-at-a-time force kernel's X table (81 slots x 128 particles x
    16 B) leaves no room for 32-row chunks, so the context takes fewer rows per chunk; the sum
    still matches the oracle."""
    p, s, a_type, r0, v = charged_system(n_kmax=40)
    g, o = gpu_and_oracle(oracle_mod, p, s, a_type, r0, v, None, "fp64")
    nk, _ = g.kspace_info()
    assert nk == len(o.kvecs())
    g.zero_force(); uk = g.ewald_k()[0]; fk = g.state()[3]
    o.zero_force(); uko = o.ewald_k(); fko = o.state()[3]
    assert rel(uk, uko) < 1e-10
    assert_force_parity(fk, fko, "fp64")


def test_ewald_contexts_with_different_tables_coexist(gpu, oracle_mod):
    """A context whose force kernel needs more shared memory (n_kmax = 17, mixed: the one-k-at-a-
    time kernel) keeps working after a second context with small tables (n_kmax = 5) is made."""
    p17, s, a_type, r0, v = charged_system(n_kmax=17)
    p5, _, _, _, _ = charged_system(n_kmax=5)
    g17 = md.MdSystem(p17, s, a_type, r0, v, precision="mixed")
    g5 = md.MdSystem(p5, s, a_type, r0, v, precision="mixed")
    o = oracle_mod.Oracle(p17, s, a_type, r0, v)
    o.ewald_init()
    g5.zero_force(); g5.ewald_k()
    g17.zero_force(); uk = g17.ewald_k()[0]; fk = g17.state()[3]
    o.zero_force(); uko = o.ewald_k(); fko = o.state()[3]
    assert rel(uk, uko) < 1e-5
    assert_force_parity(fk, fko, "mixed")
    g5.close()
    g17.close()


def charged_batch():
    """Three charged brush channels of different boxes, grafting densities and chain lengths (each
    replica gets its own k-set from its own box)."""
    p, _, _, _, _ = charged_system()
    return p, [configs.brush_channel(10.0, 10.0, 0.08, 10, rho=0.5, seed=21),
               configs.brush_channel(12.0, 9.0, 0.1, 8, rho=0.5, seed=22),
               configs.brush_channel(11.0, 11.0, 0.05, 12, rho=0.5, seed=23)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ewald_batch_matches_oracle_per_replica(gpu, oracle_mod, precision):
    """A batch of three charged replicas: the k-space energy, forces and slab dipole correction of
    each replica against its own oracle (ewald_k.f90 and dipolar_correction.f90 per system)."""
    p, reps = charged_batch()
    systems, a_type, r0, v = configs.concat(reps)
    g = md.MdSystem(p, systems, a_type, r0, v, precision=precision)
    g.zero_force(); uk = g.ewald_k(); fk = g.state()[3]
    g.zero_force(); ud = g.dipolar_correction(); fd = g.state()[3]
    off = 0
    nks = []
    for k, (s, at, rr, vv) in enumerate(reps):
        o = oracle_mod.Oracle(p, s, at, rr, vv)
        o.ewald_init()
        nks.append(len(o.kvecs()))
        o.zero_force(); uko = o.ewald_k(); fko = o.state()[3]
        o.zero_force(); udo = o.dipolar_correction(); fdo = o.state()[3]
        n = s.n_part
        assert rel(uk[k], uko) < (1e-10 if precision == "fp64" else 1e-5)
        assert_force_parity(fk[off:off + n], fko, precision)
        assert rel(ud[k], udo) < 1e-10
        assert np.abs(fd[off:off + n] - fdo).max() < 1e-10 * max(1.0, np.abs(fdo).max())
        off += n
    assert len(set(nks)) >= 2  # the replicas' boxes give different k-sets
    assert g.kspace_info()[0] == nks[0]  # mfa_kspace_info reports the first replica
    assert [g.kspace_info(k)[0] for k in range(3)] == nks
    with pytest.raises(abi.MfaError):
        g.kspace_info(3)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_charged_batch_equals_single(gpu, precision):
    """A charged replica inside a batch gets a bit-identical trajectory to the same replica run
    alone: its k-space sums cover its own charges in the same order.  Its energies agree to
    round-off (1e-12 FP64, 1e-7 mixed, whose kernels add a warp's terms in FP32 before the FP64
    totals): a batch's warps straddle the replicas' boundaries, which regroups the terms."""
    p, reps = charged_batch()
    systems, a_type, r0, v = configs.concat(reps)
    gb = md.MdSystem(p, systems, a_type, r0, v, precision=precision, nbr_capacity=160)
    gb.step(30)
    rb, vb, _, _ = gb.state()
    eb = gb.energies()
    off = 0
    for k, (s, at, rr, vv) in enumerate(reps):
        g1 = md.MdSystem(p, s, at, rr, vv, precision=precision, nbr_capacity=160)
        g1.step(30)
        r1, v1, _, _ = g1.state()
        n = s.n_part
        assert np.array_equal(r1, rb[off:off + n])
        assert np.array_equal(v1, vb[off:off + n])
        e1 = g1.energies()[0]
        for key in ("v_coul", "v_total", "e_total"):
            assert rel(e1[key], eb[k][key]) < (1e-12 if precision == "fp64" else 1e-7), key
        g1.close()
        off += n
    gb.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_charged_run_deterministic(gpu, precision):
    """A charged system (slab Ewald + dipolar correction) run twice gives bit-identical states and
    energies: every k-space sum (rho over particle chunks, U over blocks, forces over k-chunks,
    M_z) is taken in a fixed order, without floating-point atomics."""
    p, s, a_type, r0, v = charged_system()
    out = []
    for _ in range(2):
        g = md.MdSystem(p, s, a_type, r0, v, precision=precision)
        g.step(30)
        g.zero_force()
        uk = g.ewald_k()[0]
        ud = g.dipolar_correction()[0]
        out.append((uk, ud) + tuple(g.state()))
        g.close()
    assert out[0][0] == out[1][0] and out[0][1] == out[1][1]
    for x, y in zip(out[0][2:], out[1][2:]):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("block", [32, 64])
def test_pair_block_size_does_not_change_the_trajectory(gpu, block):
    """The pair kernel's block size (mfa_options.block_size, picked by the tuner) changes only the
    grouping of threads: each particle's force sums its list in the same order, so 20 fused steps
    give the same state bit for bit as the built-in 128 threads."""
    p = configs.wca_params(gamma=5.0)
    systems, a_type, r0, v = configs.concat(configs.replicas(4, seed=9))
    out = []
    for b in (128, block):
        g = md.MdSystem(p, systems, a_type, r0, v, precision="mixed", block_size=b)
        g.step(20)
        out.append(g.state())
        g.close()
    for x, y in zip(out[0], out[1]):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("setup", ["brush", "melt", "two_liquid"])
def test_energy_cadence_does_not_change_the_trajectory(gpu, setup):
    """Steps that record energies run the pair kernel's energy variant, which also forms energies
    and virial tensors from the force terms; the force terms it shares with them are rounded
    unmerged (no multiply-add whose use depends on the variant), so 30 fused steps with energies
    every step, every 10th step and every 7th step give the same state bit for bit (brush
    replicas; melt in brush with cosine bending; two liquids with the body force)."""
    if setup == "brush":
        p = configs.wca_params(gamma=5.0)
        systems, a_type, r0, v = configs.concat(configs.replicas(4, seed=9))
    elif setup == "melt":
        p, (systems, a_type, r0, v) = configs.melt_brush(L=14.0, D=24.0)
    else:
        p, _ = md.derive(configs.two_liquid_inputs(f_x=0.01))
        systems, a_type, r0, v = configs.two_liquid_channel(L=14.0, D=12.0, seed=5)
    out = []
    for every in (1, 10, 7):
        g = md.MdSystem(p, systems, a_type, r0, v, precision="mixed", energy_every=every)
        g.step(30)
        out.append(g.state())
        g.close()
    for o in out[1:]:
        for x, y in zip(out[0], o):
            assert np.array_equal(x, y)


def test_persistent_pair_schedule_does_not_change_the_trajectory(gpu):
    """mfa_options.pair_schedule 1 (persistent blocks taking 128-particle tiles from a queue)
    changes only which block evaluates a particle: 30 fused steps (rebuilds included, energies
    every 10th step) give the same state bit for bit, and the queue is reset between launches
    (a second context and a second run agree too)."""
    p = configs.wca_params(gamma=5.0)
    systems, a_type, r0, v = configs.concat(configs.replicas(6, seed=4))
    out = []
    for sch in (0, 1, 1):
        g = md.MdSystem(p, systems, a_type, r0, v, precision="mixed", pair_schedule=sch)
        g.step(30)
        out.append(g.state())
        g.close()
    for o in out[1:]:
        for x, y in zip(out[0], o):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("setup", ["brush", "melt"])
def test_fused_integration_does_not_change_the_trajectory(gpu, setup):
    """The mixed mfa_step runs the integration of its steps in the pair kernel's tail, with the
    views written to the other buffer set (options.separate_integrator 0, the default); with a
    separate integrator kernel (1) the state is the same bit for bit: over calls of 7, 13 and 10
    steps (odd and even numbers of fused steps, rebuilds and energy steps included), then a
    drop-in pair force evaluation on the views that the calls left; the energy series agrees."""
    if setup == "brush":
        p = configs.wca_params(gamma=5.0)
        systems, a_type, r0, v = configs.concat(configs.replicas(4, seed=9))
    else:
        p, (systems, a_type, r0, v) = configs.melt_brush(L=14.0, D=24.0)
    out = []
    for sep in (False, True):
        g = md.MdSystem(p, systems, a_type, r0, v, precision="mixed", separate_integrator=sep, energy_every=5,
                        series_capacity=16)
        states, series = [], []
        for n in (7, 13, 10):
            g.step(n)
            states.append(g.state())
            series += g.energy_series()
        g.zero_force()
        e = g.fluid_fluid()[0]
        out.append((states, g.state()[3], e, g.step_index(), series))
        g.close()
    (s0, f0, e0, k0, r0_), (s1, f1, e1, k1, r1_) = out
    assert k0 == k1
    for a, b in zip(s0, s1):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
    assert np.array_equal(f0, f1) and np.array_equal(e0, e1)
    # the energy records (every 5th step and the last of each call; the fused energy steps push
    # the kinetic energy and head forces from the pair kernel): same steps, same values up to the
    # order of the FP64 atomic sums
    assert len(r0_) == len(r1_) >= 6
    for a, b in zip(r0_, r1_):
        for ra, rb in zip(a, b):
            assert ra["step"] == rb["step"]
            for key in ("v_fluid_fluid", "v_intra_molec", "v_fluid_wall", "t_fluid", "e_total"):
                assert abs(ra[key] - rb[key]) <= 1e-12 * max(abs(rb[key]), 1.0), (key, ra[key], rb[key])


def test_measurement_aids(gpu):
    """mfa_fp32_fma_peak measures a plausible FP32 FMA throughput (a GB300 has 152 SMs x 128 lanes
    x 2 FLOP x ~2 GHz = ~80 TFLOP/s nominal); mfa_kspace_info gives the k-set and charge counts of
    a charged context and zeros for an uncharged one."""
    import ctypes as C
    from mfa_brush_gb300 import abi
    peak = C.c_double(0.0)
    assert abi.load_library().mfa_fp32_fma_peak(0, C.byref(peak)) == 0
    assert 10.0 < peak.value < 200.0
    assert abi.load_library().mfa_fp32_fma_peak(99, C.byref(peak)) == -1  # MFA_ERR_ARG
    p, s, a_type, r0, v = charged_system()
    g = md.MdSystem(p, s, a_type, r0, v, precision="mixed")
    nk, nq = g.kspace_info()
    assert nk > 0 and nq == int(np.count_nonzero([p.charge[t - 1] for t in a_type]))
    g.close()
    pu = configs.wca_params(gamma=5.0)
    g = md.MdSystem(pu, s, a_type, r0, v, precision="mixed")
    assert g.kspace_info() == (0, 0)
    g.close()


def test_state_round_trip_pinned_and_pageable(gpu):
    """mfa_set_state and mfa_sync_to_host move page-locked and pageable host arrays alike, one
    array at a time through the staging buffer, overlapping each copy with the previous array's
    scatter (or the next array's gather).  Both give the same state, and a round trip
    of an unchanged state is exact and needs no list rebuild."""
    torch = pytest.importorskip("torch")
    from mfa_brush_gb300 import abi
    p = configs.wca_params(gamma=5.0)
    reps = [configs.brush_channel(15.0, 12.0, 0.2, 20, seed=11),
            configs.brush_channel(18.0, 10.0, 0.15, 15, seed=12)]
    systems, a_type, r0, v = configs.concat(reps)
    g = md.MdSystem(p, systems, a_type, r0, v, precision="mixed")
    g.step(20)
    n = g.n
    pin = [torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy() for _ in range(4)]
    pag = [np.zeros((n, 3)) for _ in range(4)]
    dp = abi.dptr
    abi.check(g.lib.mfa_sync_to_host(g.ctx, dp(pin[0]), dp(pin[1]), dp(pin[2]), dp(pin[3])), g.ctx)
    abi.check(g.lib.mfa_sync_to_host(g.ctx, dp(pag[0]), dp(pag[1]), dp(pag[2]), dp(pag[3])), g.ctx)
    for x, y in zip(pin, pag):
        assert np.array_equal(x, y)
    rb = g.rebuild_count()
    abi.check(g.lib.mfa_set_state(g.ctx, dp(pin[0]), dp(pin[1]), dp(pin[2])), g.ctx)
    assert g.rebuild_count() == rb
    out = [np.zeros((n, 3)) for _ in range(3)]
    abi.check(g.lib.mfa_sync_to_host(g.ctx, dp(out[0]), dp(out[1]), dp(out[2]), None), g.ctx)
    for x, y in zip(out, pin[:3]):
        assert np.array_equal(x, y)
    # a moved state (pageable) is taken, and the lists follow it
    moved = pag[0].copy()
    moved[:, 2] += 0.0  # same z
    moved[:, 0] = (moved[:, 0] + 3.0) % np.array([s.boundary[0] for s in systems]).repeat([s.n_part for s in systems])
    g.set_state(moved, None, None)
    assert g.rebuild_count() == rb + 1
    r_back = g.state()[0]
    assert np.abs(r_back - moved).max() < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("setup", ["brush", "melt"])
def test_list_cells_give_the_same_lists(gpu, precision, setup):
    """List-build cells of the whole, a half and a third of the list cut-off (list_cells 1, 2, 3)
    walk 3^3, 5^3 and 7^3 cells, and cells of a half or a third of it along x alone (list_cells 1
    with list_cells_x 2, 3) 5 x 3 x 3 and 7 x 3 x 3; the lists hold the same pairs in another
    order.  Per replica the
    same interacting pairs and the same largest list count; pair forces equal up to the order of
    the sums (FP64 1e-12, mixed 1e-5 of F_rms); 20 steps of the fused step stay within 1e-6 sigma
    (brush replicas with one cut-off; melt in brush with per-type cut-offs)."""
    if setup == "brush":
        p = configs.wca_params(gamma=5.0)
        systems, a_type, r0, v = configs.concat(configs.replicas(4, seed=9))
        systems = list(systems)
    else:
        p, (s, a_type, r0, v) = configs.melt_brush(L=14.0, D=24.0)
        systems = [s]
    out = {}
    for h in (1, 2, 3, (1, 2), (1, 3)):
        hyz, hx = h if isinstance(h, tuple) else (h, h)
        g = md.MdSystem(p, systems, a_type, r0, v, precision=precision, list_cells=hyz, list_cells_x=hx)
        assert g.list_cells() == hyz and g.options_in_use().list_cells_x == hx
        pairs = [set(map(tuple, np.sort(g.pair_list(k), axis=1).tolist())) for k in range(len(systems))]
        g.zero_force()
        g.fluid_fluid()
        f = g.state()[3]
        mx = g.list_stats()[1]
        g.step(20)
        out[h] = (pairs, f, mx, g.state()[0])
        g.close()
    g = md.MdSystem(p, systems, a_type, r0, v, precision=precision)
    # these boxes hold three cells of the list cut-off in x and y, and five of half of it in x
    assert g.list_cells() == 1 and g.options_in_use().list_cells_x == 2
    g.close()
    pairs2, f2, mx2, r2 = out[2]
    frms = np.sqrt(np.mean(np.sum(f2 ** 2, axis=1)))
    tol = 1e-12 if precision == "fp64" else 1e-5
    for h in (1, 3, (1, 2), (1, 3)):
        pairs, f, mx, r = out[h]
        assert pairs == pairs2 and mx == mx2
        assert np.abs(f - f2).max() <= tol * frms, (h, np.abs(f - f2).max() / frms)
        d = r - r2
        L = np.concatenate([np.tile(np.array(list(s.boundary))[:2], (s.n_part, 1)) for s in systems])
        d[:, :2] -= L * np.round(d[:, :2] / L)
        assert np.abs(d).max() < 1e-6, (h, np.abs(d).max())
