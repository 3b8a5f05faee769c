"""GPU parity on the configuration families beyond the try deck, through the C ABI against the
oracle: melt chains in a brush with cosine bending on every chain (the large melt-in-brush
case), the Poiseuille body force with fixed heads (the two-liquid channel case), and the NVE
energy drift of the mixed-precision step against the FP64 oracle over 10^4 steps.

Tolerances as in test_gpu_parity.py; the drift criterion is the one the mixed mode is built to:
its energy drift within 2x of the FP64 oracle's (with a floor at the FP64 round-off level)."""
import os

import numpy as np
import pytest

from conftest import assert_force_parity
from mfa_brush_gb300 import abi, configs, md

pytestmark = pytest.mark.gpu


def rel(x, y):
    return abs(x - y) / max(abs(y), 1e-300)


def melt_brush_inputs(try_deck):
    """The try deck's switches (SOLVENT 3, brush in good solvent, DPD in the LJ range) with
    cosine bending k_b = 2 on the brush and on the melt chains."""
    inp = abi.Inputs.from_buffer_copy(try_deck[0])
    f = inp.flags
    f.bending, f.bending_melt, f.orientation = 1, 1, 0
    f.dpd_cut_off, f.force_switch_on, f.profiles = 0.0, 0, 0
    inp.bend_form, inp.k_bend = 1, 2.0
    inp.dt = 0.002
    return inp


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_melt_in_brush_cosine_bending(gpu, try_deck, oracle_mod, precision):
    inp = melt_brush_inputs(try_deck)
    p, _ = md.derive(inp)
    s, a_type, r0, v = configs.brush_channel(14.0, 12.0, 0.15, 16, rho=0.85, n_mon_d=10, seed=7, max_fill=0.75)
    assert s.n_chain_d > 0 and p.bend_form == 1
    g = md.MdSystem(p, s, a_type, r0, v, precision=precision)
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    tol_e = 1e-10 if precision == "fp64" else 1e-5
    # each routine's energy; the forces summed over the four routines, as md_main sums them.
    # (A bending force alone on a nearly straight chain is ~sin(angle) small and its FP32
    # direction carries a relative error ~1e-7/angle; only max|dF|/F_rms is asked of it.)
    g.zero_force()
    o.zero_force()
    for routine, key in (("fluid_fluid", "v_fluid_fluid"), ("intra_molec", "v_intra_molec"),
                         ("bending", "v_bend"), ("bending_melt", "v_bend_melt")):
        f0, fo0 = g.state()[3], o.state()[3]
        e = getattr(g, routine)()
        e = e[0] if isinstance(e, tuple) else e
        getattr(o, routine)()
        assert rel(e[0], o.energies()[key]) < tol_e, routine
        df, dfo = g.state()[3] - f0, o.state()[3] - fo0
        rms = np.sqrt(np.mean(np.sum(dfo ** 2, axis=1)))
        assert np.linalg.norm(df - dfo, axis=1).max() <= (1e-9 if precision == "fp64" else 1e-5) * rms, routine
    assert_force_parity(g.state()[3], o.state()[3], precision)


def test_melt_in_brush_fused_mixed_steps(gpu, try_deck, oracle_mod):
    inp = melt_brush_inputs(try_deck)
    p, _ = md.derive(inp)
    s, a_type, r0, v = configs.brush_channel(14.0, 12.0, 0.15, 16, rho=0.85, n_mon_d=10, seed=8, max_fill=0.75)
    g = md.MdSystem(p, s, a_type, r0, v, precision="mixed")
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    g.step(10)
    o.step(10, 1, 0)
    r, vv, _, _ = g.state()
    ro, vo, _, _ = o.state()
    L = np.array(list(s.boundary))
    d = r - ro
    d[:, :2] -= L[:2] * np.round(d[:, :2] / L[:2])
    assert np.abs(d).max() < 1e-7
    assert np.abs(vv - vo).max() < 1e-4 * np.sqrt(np.mean(vo ** 2))
    eg, eo = g.energies()[0], o.energies()
    for k in ("v_fluid_fluid", "v_intra_molec", "v_bend", "v_bend_melt", "t_fluid"):
        assert rel(eg[k], eo[k]) < 1e-5, k


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_poiseuille_body_force_and_fixed_heads(gpu, try_deck, oracle_mod, precision):
    """POISEUILLE: m g on every non-head bead (constant_force.f90:17-21) and heads held at rest
    (verlet_velocities.f90:115-120); five md_main steps through the drop-ins (FP64) or the fused
    step (mixed) against the oracle."""
    inp = abi.Inputs.from_buffer_copy(try_deck[0])
    inp.flags.poiseuille = 1
    inp.const_force[0], inp.const_force[1], inp.const_force[2] = 0.05, 0.0, 0.0
    p, s = md.derive(inp)
    _, _, _, a_type, r0, v, a = try_deck
    g = md.MdSystem(p, s, a_type, r0, v, a, precision=precision)
    o = oracle_mod.Oracle(p, s, a_type, r0, v, a)
    if precision == "fp64":
        for _ in range(5):
            g.md_step()
    else:
        g.step(5)
    o.step(5, 1, 0)
    r, vv, _, _ = g.state()
    ro, vo, _, _ = o.state()
    L = np.array(list(s.boundary))
    d = r - ro
    d[:, :2] -= L[:2] * np.round(d[:, :2] / L[:2])
    assert np.abs(d).max() < (1e-9 if precision == "fp64" else 1e-7)
    heads = np.flatnonzero(a_type == 1)
    assert np.abs(vv[heads]).max() == 0.0
    tol = 1e-7 if precision == "fp64" else 1e-4
    assert np.abs(vv - vo).max() < tol * max(1.0, np.sqrt(np.mean(vo ** 2)))


def _energy_series(run, n_steps, every):
    e = []
    for _ in range(n_steps // every):
        e.append(run(every))
    return np.array(e)


def test_nve_drift_mixed_within_2x_fp64_oracle(gpu, oracle_mod):
    """10^4 NVE steps (no thermostat) of a WCA brush channel: the mixed-precision total-energy
    drift (slope of a linear fit, per particle per step) stays within 2x of the FP64 oracle's."""
    p = configs.wca_params(gamma=0.0, thermostat=1, dt=0.005)
    s, a_type, r0, v = configs.brush_channel(12.0, 10.0, 0.15, 12, seed=31, kT=0.5)
    n, every = 10000, 500
    g = md.MdSystem(p, s, a_type, r0, v, precision="mixed")
    o = oracle_mod.Oracle(p, s, a_type, r0, v)

    def run_g(k):
        g.step(k)
        return g.energies()[0]["e_total"]

    threads = max(1, os.cpu_count() or 1)

    def run_o(k):
        o.step(k, threads, 0)
        e = o.energies()
        return e["v_fluid_fluid"] + e["v_fluid_wall"] + e["v_wall_wall"] + e["v_intra_molec"] + e["t_fluid"]

    eg = _energy_series(run_g, n, every)
    eo = _energy_series(run_o, n, every)
    t = np.arange(1, len(eg) + 1) * every
    slope_g = abs(np.polyfit(t, eg, 1)[0]) / s.n_mon_tot
    slope_o = abs(np.polyfit(t, eo, 1)[0]) / s.n_mon_tot
    print("NVE drift per particle per step: mixed %.3e  fp64 oracle %.3e" % (slope_g, slope_o))
    assert np.all(np.isfinite(eg))
    assert slope_g <= 2.0 * max(slope_o, 1e-9)


def test_charged_nve_energy_excursion_within_3x_fp64_oracle(gpu, oracle_mod):
    """2000 NVE steps (no thermostat) of a strongly charged brush channel (brush beads -1, solvent
    +1, slab Ewald, dipolar correction) through the fused mixed-precision step: the total energy,
    Coulomb terms included, starts where the FP64 oracle's does, and its largest excursion from
    the start stays within 3x of the oracle's (or 1e-5 of |E|)."""
    inp = configs.wca_inputs(gamma=0.0, thermostat=1)
    inp.flags.system = 3
    inp.charge[1], inp.charge[2] = -1.0, 1.0
    inp.alpha_c, inp.n_kmax, inp.rc_coul = 0.81, 5, 3.0
    p, _ = md.derive(inp)
    s, a_type, r0, v = configs.brush_channel(10.0, 10.0, 0.08, 10, rho=0.5, seed=21, kT=0.5, max_fill=0.75)
    n, every = 2000, 200
    g = md.MdSystem(p, s, a_type, r0, v, precision="mixed")
    o = oracle_mod.Oracle(p, s, a_type, r0, v)

    def run_g(k):
        g.step(k)
        return g.energies()[0]["e_total"]

    threads = max(1, os.cpu_count() or 1)

    def run_o(k):
        o.step(k, threads, 0)
        return sum(o.energies().values())

    eg = _energy_series(run_g, n, every)
    eo = _energy_series(run_o, n, every)
    dg = np.abs(eg - eg[0]).max()
    do = np.abs(eo - eo[0]).max()
    print("charged NVE, %d steps: E %.4f (mixed) %.4f (fp64 oracle); largest excursion %.3e / %.3e"
          % (n, eg[0], eo[0], dg, do))
    assert np.all(np.isfinite(eg))
    assert abs(eg[0] - eo[0]) < 1e-3 * abs(eo[0])
    assert dg <= 3.0 * max(do, 1e-5 * abs(eo[0]))


def test_dpd_statistics_match_oracle(gpu, oracle_mod):
    """With the DPD noise on, the fused mixed step samples the same process as FP64.  WCA channel
    10 x 10 x 10 sigma with 12-bead chains, DPD with its own 1.5 sigma cut-off, kT = 1: 1500 steps
    of equilibration, then 60 samples 100 steps apart of the kinetic temperature, the velocity
    kurtosis (3 for a Maxwell distribution), the brush height (mean distance of the brush beads
    from their own wall) and the solvent z-profile.
    (1) Eight independent replicas (own starts, own Philox keys) run batched on the mixed path and
    on the FP64 path; their per-replica means agree within 5 standard errors over the replicas
    (the brush height relaxes over thousands of steps, so the samples of one trajectory are far
    from independent; the replicas are).
    (2) The oracle runs the first replica (the same start and Philox stream; the trajectories part
    after a few hundred steps): its temperature and kurtosis are the Maxwell values, and its brush
    height and profile lie within the spread of the GPU replicas."""
    inp = configs.wca_inputs(gamma=5.0, kT=1.0, dt=0.005)
    inp.flags.dpd_cut_off = 1.5  # DPD_CUT_OFF
    p, _ = md.derive(inp)
    reps = [configs.brush_channel(10.0, 10.0, 0.15, 12, rho=0.7, seed=13 + k) for k in range(8)]
    systems, a_type, r0, v = configs.concat(reps)

    def sample(s, at, r, vv):
        nb, D = s.n_mon * s.n_chain, s.boundary[2]
        vm = vv[at != 1]
        t = np.mean(vm ** 2)
        k4 = np.mean(vm ** 4) / t ** 2
        bottom = np.zeros(s.n_part, bool)
        bottom[: (s.n_chain // 2) * s.n_mon] = True  # the first half of the chains hang from z = 0
        brush = at == 2
        h = np.mean(np.where(bottom[brush], r[brush, 2], D - r[brush, 2]))
        prof = np.histogram(r[nb:, 2], bins=10, range=(0.0, D))[0].astype(float)
        return np.concatenate([[t, k4, h], prof / prof.sum()])

    def replica_means(precision):
        g = md.MdSystem(p, systems, a_type, r0, v, precision=precision)
        g.step(1500)
        acc = []
        for _ in range(60):
            g.step(100)
            r, vv = g.state()[:2]
            row, off = [], 0
            for s, at, _, _ in reps:
                sl = slice(off, off + s.n_part)
                row.append(sample(s, at, r[sl], vv[sl]))
                off += s.n_part
            acc.append(row)
        g.close()
        return np.mean(np.array(acc), axis=0)  # (replica, observable)

    mix, f64 = replica_means("mixed"), replica_means("fp64")
    se = np.hypot(mix.std(axis=0, ddof=1), f64.std(axis=0, ddof=1)) / np.sqrt(len(reps))
    dm = np.abs(mix.mean(axis=0) - f64.mean(axis=0))
    prof_l1 = np.abs(mix[:, 3:].mean(axis=0) - f64[:, 3:].mean(axis=0)).sum()
    print("DPD statistics over %d replicas, mixed / FP64: <v^2> %.4f / %.4f  kurtosis %.3f / %.3f  "
          "brush height %.3f / %.3f (standard error %.3f)  profile L1 %.4f"
          % (len(reps), mix[:, 0].mean(), f64[:, 0].mean(), mix[:, 1].mean(), f64[:, 1].mean(),
             mix[:, 2].mean(), f64[:, 2].mean(), se[2], prof_l1))
    assert np.all(np.abs(mix[:, 0] - 1.0) < 0.05) and np.all(np.abs(f64[:, 0] - 1.0) < 0.05)
    for c in range(len(dm)):  # temperature, kurtosis, brush height, the ten profile bins
        assert dm[c] < 5 * se[c] + 1e-3, (c, dm[c], se[c])
    assert prof_l1 < 0.04

    s, at, r, vv = reps[0]
    o = oracle_mod.Oracle(p, s, at, r, vv)
    threads = max(1, os.cpu_count() or 1)
    o.step(1500, threads, 0)
    so = []
    for _ in range(60):
        o.step(100, threads, 0)
        so.append(sample(s, at, *o.state()[:2]))
    o.close()
    so = np.mean(np.array(so), axis=0)
    pool = np.concatenate([mix, f64])
    spread = pool.std(axis=0, ddof=1)
    print("oracle, replica 0: <v^2> %.4f  kurtosis %.3f  brush height %.3f (GPU replicas %.3f +- %.3f)  "
          "profile L1 to the GPU mean %.4f" % (so[0], so[1], so[2], pool[:, 2].mean(), spread[2],
                                               np.abs(so[3:] - pool[:, 3:].mean(axis=0)).sum()))
    assert abs(so[0] - 1.0) < 0.05 and abs(so[1] - 3.0) < 0.1
    assert abs(so[2] - pool[:, 2].mean()) < 4 * spread[2] + 1e-3
    assert np.abs(so[3:] - pool[:, 3:].mean(axis=0)).sum() < 0.08


def test_charged_brush_full_size_stays_in_channel(gpu):
    """The full-size charged brush (33,600 particles, 1280 counterions, 8070 k-vectors) for 300
    fused mixed steps under the DPD thermostat: every particle stays in the channel and the
    energies stay finite.  The lattice start releases heat that the DPD thermostat, acting inside
    the WCA range only, removes over ~10^3 steps.  The FP64 oracle on the same system and noise
    has <v^2> = 1.767 per component at step 300 (its 300 steps take ~25 minutes on 8 cores, so
    the value is written here); the mixed run must agree within 0.06."""
    p, (s, a_type, r0, v) = configs.charged_brush()
    g = md.MdSystem(p, s, a_type, r0, v, precision="mixed")
    g.step(300)
    r, vv, _, _ = g.state()
    e = g.energies()[0]
    g.close()
    assert np.all(np.isfinite(r)) and np.all(np.isfinite(vv))
    assert r[:, 2].min() > 0.0 and r[:, 2].max() < s.boundary[2]
    mob = a_type != 1
    t_kin = np.mean(vv[mob] ** 2)
    print("charged brush after 300 steps: <v^2> per component %.3f, e_total %.1f" % (t_kin, e["e_total"]))
    assert abs(t_kin - 1.767) < 0.06
    assert np.isfinite(e["e_total"])


@pytest.mark.parametrize("model", ["counterions", "uniform"])
def test_charged_brush_kspace_precision_at_full_size(gpu, oracle_mod, model):
    """The charged-brush case at its full size: 40 x 40 x 30 channel, grafting density 0.1, N = 40,
    slab Ewald with alpha = 0.9 (alpha_c = 0.81), real-space cut-off 3, |k| <= 12 (2 pi / L) with
    the reference's k-set rule (8070 vectors), dipolar correction.  "counterions": the brush charge
    -4 per chain spread over its beads, 1280 +1 counterions, neutral solvent (13,760 charged
    particles; configs.charged_brush).  "uniform": -0.1 per brush bead neutralised by the whole
    solvent (33,280 charged particles).  Prints the k-space energy, force and virial errors of the
    FP64, the mixed (Kahan-compensated FP32) and the plain FP32 sums against the FP64 oracle; the
    mixed path must meet the 1e-5 criterion on each."""
    if model == "counterions":
        p, (s, a_type, r0, v) = configs.charged_brush(gamma=1.0)
    else:
        s, a_type, r0, v = configs.brush_channel(40.0, 30.0, 0.1, 40, rho=0.7, seed=41)
        n_brush = int(np.sum(a_type == 2))
        n_solv = int(np.sum(a_type == 3))
        inp = configs.wca_inputs(gamma=1.0, thermostat=0)
        inp.flags.system = 3
        inp.charge[1] = -0.1
        inp.charge[2] = 0.1 * n_brush / n_solv
        inp.alpha_c = 0.81
        inp.n_kmax = 12
        inp.rc_coul = 3.0
        p, _ = md.derive(inp)
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    o.ewald_init()
    o.zero_force()
    uko = o.ewald_k()
    fko = o.state()[3]
    wko = o.virial()["kspace"]
    rms = np.sqrt(np.mean(np.sum(fko ** 2, axis=1)))
    out = {}
    for name, precision, plain in (("fp64", "fp64", False), ("mixed", "mixed", False), ("plain", "mixed", True)):
        g = md.MdSystem(p, s, a_type, r0, v, precision=precision, kspace_plain_sums=plain)
        g.zero_force()
        uk = g.ewald_k()[0]
        fk = g.state()[3]
        wk = g.virial()[0]["kspace"]
        out[name] = (rel(uk, uko), np.linalg.norm(fk - fko, axis=1).max() / rms,
                     np.abs(wk - wko).max() / np.abs(wko).max())
        g.close()
    print("k-space vs FP64 oracle (%s, N=%d; rel energy error, max|dF|/F_rms, max|dW|/max|W| of the "
          "k-space virial): fp64 %.2e %.2e %.2e  compensated FP32 %.2e %.2e %.2e  plain FP32 %.2e %.2e %.2e"
          % (model, s.n_mon_tot, *out["fp64"], *out["mixed"], *out["plain"]))
    assert out["fp64"][0] < 1e-10 and out["fp64"][1] < 1e-9 and out["fp64"][2] < 1e-10
    assert out["mixed"][0] < 1e-5 and out["mixed"][1] < 1e-5 and out["mixed"][2] < 1e-5
    assert out["plain"][0] < 1e-3 and out["plain"][1] < 1e-3  # reported; no 1e-5 promise


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_two_liquid_poiseuille_channel(gpu, oracle_mod, precision):
    """The two-liquid Poiseuille family: liquids A (type 3) and B (type 4, PARTICLE_4) in layered
    halves, eps_AB = 0.5, every liquid pair cut at 2 * 2^(1/6), brush WCA, body force f_x on every
    non-head bead, z-profiles of three species.  Pair + wall + body forces against the oracle,
    then six steps with profiles (drop-ins in FP64, the fused graph step in mixed)."""
    inp = configs.two_liquid_inputs(f_x=0.05)
    p, _ = md.derive(inp)
    s, a_type, r0, v = configs.two_liquid_channel(seed=3)
    g = md.MdSystem(p, s, a_type, r0, v, precision=precision, profile_from_step=0)
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    g.zero_force()
    vff = g.fluid_fluid()[0][0]
    vfw = g.fluid_wall(2)[0]
    g.constant_force(1)
    o.zero_force()
    o.fluid_fluid()
    o.fluid_wall()
    o.constant_force()
    eo = o.energies()
    tol_e = 1e-10 if precision == "fp64" else 1e-5
    assert rel(vff, eo["v_fluid_fluid"]) < tol_e and rel(vfw, eo["v_fluid_wall"]) < 1e-10
    assert_force_parity(g.state()[3], o.state()[3], precision)
    g.reset_profiles()
    if precision == "fp64":
        for _ in range(6):
            g.md_step(profiles=True)
    else:
        g.step(6)
    o.step(6, 1, 1)
    dg, vg, v2g, ng = g.profiles(0)
    do, vo, v2o, no = o.profiles()
    assert ng == no == 6
    assert dg.reshape(-1, 3).sum(0)[1:].tolist() == do.reshape(-1, 3).sum(0)[1:].tolist()  # A, B counts
    if precision == "fp64":
        assert np.array_equal(dg, do)
        assert np.abs(vg - vo).max() < 1e-9 and np.abs(v2g - v2o).max() < 1e-9
    else:
        # a bead within ~1e-7 sigma of a bin edge may land in the neighbouring bin
        assert np.abs(dg - do).sum() <= 8
        assert np.abs(vg.sum(0) - vo.sum(0)).max() < 1e-3 * max(1.0, np.abs(vo).sum())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_observation_quantities(gpu, try_deck, oracle_mod, precision):
    """mfa_observe against the oracle's observation.f90 restatement after five steps: brush and
    melt Rg^2 per axis, total momentum, and the summed head forces of the last velocity step."""
    inp = melt_brush_inputs(try_deck)
    p, _ = md.derive(inp)
    s, a_type, r0, v = configs.brush_channel(14.0, 12.0, 0.15, 16, rho=0.85, n_mon_d=10, seed=9, max_fill=0.75)
    g = md.MdSystem(p, s, a_type, r0, v, precision=precision)
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    if precision == "fp64":
        for _ in range(5):
            g.md_step()
    else:
        g.step(5)
    o.step(5, 1, 0)
    og, oo = g.observe()[0], o.observe()
    tol = 1e-9 if precision == "fp64" else 1e-6
    for key in ("rg2_brush", "rg2_melt"):
        assert np.allclose(og[key], oo[key], rtol=tol, atol=0), key
    m = np.array([p.mass_type[t - 1] for t in a_type[: s.n_mon_tot]])
    scale = np.abs(m[:, None] * o.state()[1][: s.n_mon_tot]).sum()
    assert np.abs(np.array(og["momentum"]) - np.array(oo["momentum"])).max() < tol * scale
    fh, fo = np.array(og["f_heads"]), np.array(oo["f_heads"])
    assert np.abs(fh - fo).max() < (1e-9 if precision == "fp64" else 1e-5) * np.abs(fo).max()


def test_ragged_batch_edge_cases(gpu, oracle_mod):
    """A batch of a pure-solvent replica, a one-chain-per-wall replica and a short-box replica:
    every replica against its own FP64 oracle after five drop-in steps, and the same batch built
    with a list capacity far too small (the context grows it at start-up)."""
    p = configs.wca_params(gamma=5.0)
    reps = [configs.brush_channel(10.0, 8.0, 0.0, 10, seed=51),
            configs.brush_channel(12.0, 10.0, 1.0 / 144.0, 25, seed=52),
            configs.brush_channel(7.5, 12.0, 0.2, 8, seed=53)]
    assert reps[0][0].n_chain == 0 and reps[1][0].n_chain == 2
    systems, a_type, r0, v = configs.concat(reps)
    for cap in (0, 4):
        g = md.MdSystem(p, systems, a_type, r0, v, precision="fp64", nbr_capacity=cap)
        for _ in range(5):
            g.md_step()
        r, vv, _, _ = g.state()
        off = 0
        for (s, at, rr, v0) in reps:
            o = oracle_mod.Oracle(p, s, at, rr, v0)
            o.step(5, 1, 0)
            ro, vo, _, _ = o.state()
            n = s.n_part
            L = np.array(list(s.boundary))
            d = r[off:off + n] - ro
            d[:, :2] -= L[:2] * np.round(d[:, :2] / L[:2])
            assert np.abs(d).max() < 1e-9
            assert np.abs(vv[off:off + n] - vo).max() < 1e-7 * max(1.0, np.abs(vo).max())
            off += n
        assert g.step_index() == 1 + 5
        g.step(0)  # no-op
        g.close()


def test_invalid_systems_are_refused(gpu):
    p = configs.wca_params(gamma=5.0)
    s, a_type, r0, v = configs.brush_channel(10.0, 8.0, 0.1, 10, seed=54)
    bad = abi.System.from_buffer_copy(s)
    bad.boundary[0] = bad.boundary[1] = 2.0  # shorter than 2.5 list cut-offs
    with pytest.raises(abi.MfaError) as e:
        md.MdSystem(p, bad, a_type, r0, v)
    assert e.value.code == -9  # MFA_ERR_UNSUPPORTED
    bad = abi.System.from_buffer_copy(s)
    bad.n_mon_tot = s.n_mon_tot - 1  # inconsistent with the chain counts
    with pytest.raises(abi.MfaError):
        md.MdSystem(p, bad, a_type, r0, v)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_restart_continues_the_noise_stream(gpu, precision):
    """Ten steps, the state taken out, a new context started at the next step with that state, ten
    more steps: the same trajectory as twenty uninterrupted steps (the DPD noise is keyed on the
    step, so no generator state needs saving).  Agreement to round-off: the new context sorts its
    particles afresh, which changes the order of the force sums."""
    p = configs.wca_params(gamma=5.0)
    s, a_type, r0, v = configs.brush_channel(14.0, 12.0, 0.2, 20, seed=61)
    g = md.MdSystem(p, s, a_type, r0, v, precision=precision)
    g.step(20)
    r20, v20, _, _ = g.state()
    g.close()
    g = md.MdSystem(p, s, a_type, r0, v, precision=precision)
    g.step(10)
    r10, v10, a10, _ = g.state()
    g.close()
    s2 = abi.System.from_buffer_copy(s)
    s2.s_time = s.s_time + 10
    g = md.MdSystem(p, s2, a_type, r10, v10, a10, precision=precision)
    g.step(10)
    rr, vv, _, _ = g.state()
    L = np.array(list(s.boundary))
    d = rr - r20
    d[:, :2] -= L[:2] * np.round(d[:, :2] / L[:2])
    tol = 1e-10 if precision == "fp64" else 1e-5
    assert np.abs(d).max() < tol
    assert np.abs(vv - v20).max() < tol * 100


def test_list_capacity_grows_before_it_overflows(gpu):
    """A context made with a list capacity just above the largest count raises the capacity at its
    first step (the count is past 85 % of it) and then runs exactly like one with ample room."""
    p = configs.wca_params(gamma=5.0)
    s, a_type, r0, v = configs.brush_channel(14.0, 12.0, 0.2, 20, seed=71)
    ref = md.MdSystem(p, s, a_type, r0, v, precision="fp64")
    cap0, mx0 = ref.list_stats()
    assert 0 < mx0 < cap0
    tight = md.MdSystem(p, s, a_type, r0, v, precision="fp64", nbr_capacity=mx0 + 1)
    assert tight.list_stats() == (mx0 + 1, mx0)
    tight.step(30)
    ref.step(30)
    cap1, mx1 = tight.list_stats()
    assert cap1 > mx0 + 1 and mx1 <= cap1
    for x, y in zip(tight.state(), ref.state()):
        assert np.array_equal(x, y)


def test_list_overflow_is_cleared_by_the_growth(gpu):
    """A state whose lists do not fit the capacity is reported (MFA_ERR_NLIST_OVERFLOW).  After the
    original state is put back, mfa_step alone (no status-reading call in between) raises the
    capacity, rebuilds the lists and clears the overflow: the status is clean again and the
    trajectory equals that of a context with ample room."""
    p = configs.wca_params(gamma=5.0)
    s, a_type, r0, v = configs.brush_channel(14.0, 12.0, 0.2, 20, seed=71)
    ref = md.MdSystem(p, s, a_type, r0, v, precision="fp64")
    cap0, mx0 = ref.list_stats()
    cap = int(np.ceil(mx0 / 0.85)) + 2  # no growth pending after start-up
    g = md.MdSystem(p, s, a_type, r0, v, precision="fp64", nbr_capacity=cap)
    assert g.list_stats() == (cap, mx0)
    squeezed = np.array(r0, np.float64).reshape(-1, 3).copy()
    D = s.boundary[2]
    squeezed[:, 2] = 0.5 * D + 0.5 * (squeezed[:, 2] - 0.5 * D)  # twice the density: more neighbours
    with pytest.raises(abi.MfaError) as ei:
        g.set_state(r0=squeezed)
    assert abi.ERRORS[ei.value.code] == "MFA_ERR_NLIST_OVERFLOW"
    with pytest.raises(abi.MfaError):  # the rebuild of the original state fits, the overflow is still set
        g.set_state(r0=r0)
    for _ in range(3):
        g.step(10)  # the first call raises the capacity and rebuilds before its steps
    ref.step(30)
    cap1, mx1 = g.list_stats()  # would raise if the overflow bit were still set
    assert cap1 > cap and mx1 <= cap1
    for x, y in zip(g.state(), ref.state()):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_force_switch_on_ramp(gpu, try_deck, oracle_mod, precision):
    """FORCE_SWITCH_ON from s_time = 1 (init_force_switch_on.f90:12-28, fluid_fluid.f90:35-42):
    pair distances are clamped at a radius that shrinks with time.  Pair forces at the first step
    and three md_main steps against the oracle."""
    import ctypes as C
    inp, p, s, a_type, r0, v, a = try_deck
    p1 = abi.Params.from_buffer_copy(p)
    abi.check(md._lib().mfa_force_switch_on(C.byref(p1), 10000, 0))
    assert p1.r_2_min_init > 0.5 and p1.r_2_min_time >= 40.0
    s1 = abi.System.from_buffer_copy(s)
    s1.s_time = 1
    g = md.MdSystem(p1, s1, a_type, r0, v, a, precision=precision)
    o = oracle_mod.Oracle(p1, s1, a_type, r0, v, a)
    g.zero_force()
    vff = g.fluid_fluid()[0][0]
    o.zero_force()
    o.fluid_fluid()
    assert rel(vff, o.energies()["v_fluid_fluid"]) < (1e-10 if precision == "fp64" else 1e-5)
    assert abs(vff - (-1131.60193205932)) > 1.0  # the clamp is active (unclamped: the try/log value)
    assert_force_parity(g.state()[3], o.state()[3], precision)
    if precision == "fp64":
        for _ in range(3):
            g.md_step()
        o.step(3, 1, 0)
        d = g.state()[0] - o.state()[0]
        L = np.array(list(s.boundary))
        d[:, :2] -= L[:2] * np.round(d[:, :2] / L[:2])
        assert np.abs(d).max() < 1e-9


@pytest.mark.parametrize("compat", [1, 4, 5])  # MFA_COMPAT_EWALD_INV_PI, MFA_COMPAT_COUL_IN_LJ, both
def test_reference_defect_switches(gpu, oracle_mod, compat):
    """The reference's Ewald defects reproduced behind compat bits: 1/pi for 1/sqrt(pi)
    (init_config.f90:232) and real-space Coulomb only inside the LJ cut-off (fluid_fluid.f90:
    203-209).  Real-space forces and energy, FP64, against the oracle with the same bits; the
    forces (and, for the shorter range, the energy) must differ from the corrected ones."""
    def system(bits):
        inp = configs.wca_inputs(gamma=1.0, thermostat=0)
        inp.flags.system = 3
        inp.charge[1], inp.charge[2] = -1.0, 1.0
        inp.alpha_c, inp.n_kmax, inp.rc_coul = 0.81, 4, 3.0
        inp.compat = bits
        p, _ = md.derive(inp)
        return p
    s, a_type, r0, v = configs.brush_channel(10.0, 10.0, 0.08, 10, rho=0.5, seed=22)
    out = {}
    for bits in (0, compat):
        p = system(bits)
        g = md.MdSystem(p, s, a_type, r0, v, precision="fp64")
        o = oracle_mod.Oracle(p, s, a_type, r0, v)
        g.zero_force()
        _, vc = g.fluid_fluid()
        o.zero_force()
        o.fluid_fluid()
        assert abs(vc[0] - o.energies()["v_coul"]) < 1e-10 * abs(o.energies()["v_coul"])
        f = g.state()[3]
        assert_force_parity(f, o.state()[3], "fp64")
        out[bits] = (vc[0], f)
        g.close()
    # 1/pi only scales the force's Gaussian term; the shorter Coulomb range changes both
    assert np.abs(out[compat][1] - out[0][1]).max() > 1e-6 * np.abs(out[0][1]).max()
    if compat & 4:
        assert abs(out[compat][0] - out[0][0]) > 1e-6 * abs(out[0][0])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sheared_brushes_moving_heads(gpu, oracle_mod, precision):
    """Brush-brush shear (verlet_velocities.f90:111-124): the heads of chains 1..n_chain/2 move at
    va_spring_twall(1:2), the others at minus it, with no z motion; DPD on.  Twelve md_main steps
    through the drop-ins (FP64) or the fused step (mixed) against the oracle, positions,
    velocities and the kinetic energy (which counts the heads' motion); the heads advance by
    exactly +-va dt per step (modulo the box)."""
    inp = configs.wca_inputs(gamma=5.0, kT=1.0, dt=0.005)
    inp.va_spring_twall[0], inp.va_spring_twall[1], inp.va_spring_twall[2] = 0.4, -0.15, 0.0
    p, _ = md.derive(inp)
    assert tuple(p.va_wall) == (0.4, -0.15)
    s, a_type, r0, v = configs.brush_channel(12.0, 10.0, 0.15, 12, seed=17)
    g = md.MdSystem(p, s, a_type, r0, v, precision=precision)
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    n = 12
    if precision == "fp64":
        for _ in range(n):
            eg = g.md_step()[0]
    else:
        g.step(n)
        eg = g.energies()[0]
    o.step(n, 1, 0)
    r, vv, _, _ = g.state()
    ro, vo, _, _ = o.state()
    L = np.array(list(s.boundary))
    d = r - ro
    d[:, :2] -= L[:2] * np.round(d[:, :2] / L[:2])
    assert np.abs(d).max() < (1e-9 if precision == "fp64" else 1e-7)
    tol = 1e-7 if precision == "fp64" else 1e-4
    assert np.abs(vv - vo).max() < tol * max(1.0, np.sqrt(np.mean(vo ** 2)))
    heads = np.arange(s.n_chain) * s.n_mon
    sg = np.where(np.arange(s.n_chain) < s.n_chain // 2, 1.0, -1.0)
    assert np.array_equal(vv[heads, 0], sg * 0.4) and np.array_equal(vv[heads, 1], sg * -0.15)
    assert np.all(vv[heads, 2] == 0.0)
    # the first position update used the start's head velocities (zero), the other n - 1 the wall's
    dh = r[heads] - r0.reshape(-1, 3)[heads]
    dh[:, :2] -= L[:2] * np.round(dh[:, :2] / L[:2])
    want = np.stack([sg * 0.4, sg * -0.15, 0.0 * sg], axis=1) * (n - 1) * p.dt
    assert np.abs(dh - want).max() < 1e-9
    assert abs(eg["t_fluid"] - o.energies()["t_fluid"]) < (1e-9 if precision == "fp64" else 1e-5) * o.energies()["t_fluid"]
    g.close()
    o.close()


@pytest.mark.parametrize("precision", ["fp64", "fp64_fused", "mixed"])
def test_moving_explicit_walls(gpu, oracle_mod, precision):
    """Couette with explicit walls (WALL 1, verlet_positions.f90:214-247): the sites of wall beads
    1..n_wall/2 move by +va dt per step, the others by -va dt, and the heads move at +-va
    (verlet_velocities.f90:111-124).  At va = 1 the walls pass half the skin within the run, so
    the lists must be rebuilt for them.  60 md_main steps through the drop-ins (FP64) or the
    fused step (mixed, and FP64 through its fused integrator) against the oracle: the wall beads'
    positions bit for bit, the mobile particles' within the usual tolerances."""
    inp = configs.wca_inputs(gamma=5.0, wall=1, dpd_cut_off=1.0)
    inp.va_spring_twall[0], inp.va_spring_twall[1] = 1.0, -0.5
    p, _ = md.derive(inp)
    s, a_type, r0, v = configs.explicit_wall_channel(seed=8)
    fused = precision == "fp64_fused"
    precision = "fp64" if fused else precision
    g = md.MdSystem(p, s, a_type, r0, v, precision=precision)
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    n = 60
    assert n * p.dt * 1.0 > 0.5 * g.options_in_use().skin
    if precision == "fp64" and not fused:
        for _ in range(n):
            g.md_step()
    else:
        g.step(n)
    o.step(n, 1, 0)
    r, vv, _, _ = g.state()
    ro, vo, _, _ = o.state()
    nm = s.n_mon_tot
    assert np.array_equal(r[nm:], ro[nm:])
    assert np.all(vv[nm:] == 0.0)
    L = np.array(list(s.boundary))
    d = r[:nm] - ro[:nm]
    d[:, :2] -= L[:2] * np.round(d[:, :2] / L[:2])
    assert np.abs(d).max() < (1e-8 if precision == "fp64" else 1e-5)
    tol = 1e-6 if precision == "fp64" else 1e-3
    assert np.abs(vv[:nm] - vo[:nm]).max() < tol * max(1.0, np.sqrt(np.mean(vo[:nm] ** 2)))
    assert g.replica_rebuild_counts()[0] >= 1
    g.close()
    o.close()


def test_sheared_batch_equals_single(gpu):
    """Sheared brushes in a batch: each replica's heads take the wall velocity by its own chain
    count (chains 1..n_chain/2 of the replica at +va), so three replicas of different sizes run
    batched give the same trajectories, bit for bit, as each run alone (mixed, 40 fused steps)."""
    inp = configs.wca_inputs(gamma=5.0, kT=1.0, dt=0.005)
    inp.va_spring_twall[0], inp.va_spring_twall[1] = 0.3, 0.1
    p, _ = md.derive(inp)
    reps = [configs.brush_channel(12.0, 10.0, 0.15, 12, seed=31),
            configs.brush_channel(14.0, 12.0, 0.1, 20, seed=32),
            configs.brush_channel(10.0, 9.0, 0.2, 8, seed=33)]
    systems, a_type, r0, v = configs.concat(reps)
    gb = md.MdSystem(p, systems, a_type, r0, v, precision="mixed", nbr_capacity=160)
    gb.step(40)
    rb, vb, _, _ = gb.state()
    gb.close()
    off = 0
    for s, at, rr, vv in reps:
        g1 = md.MdSystem(p, s, at, rr, vv, precision="mixed", nbr_capacity=160)
        g1.step(40)
        r1, v1, _, _ = g1.state()
        g1.close()
        n = s.n_part
        assert np.array_equal(r1, rb[off:off + n]) and np.array_equal(v1, vb[off:off + n])
        heads = np.arange(s.n_chain) * s.n_mon
        sg = np.where(np.arange(s.n_chain) < s.n_chain // 2, 1.0, -1.0)
        assert np.array_equal(v1[heads, 0], 0.3 * sg)
        off += n


def test_moving_walls_batch_equals_single(gpu):
    """Moving explicit walls in a batch: each replica's wall beads 1..n_wall/2 of its own count
    move at +va, so two replicas of different sizes run batched give the same trajectories, bit
    for bit, as each run alone (mixed, 40 fused steps, the walls passing half the skin)."""
    inp = configs.wca_inputs(gamma=5.0, wall=1, dpd_cut_off=1.0)
    inp.va_spring_twall[0], inp.va_spring_twall[1] = 1.0, 0.5
    p, _ = md.derive(inp)
    reps = [configs.explicit_wall_channel(seed=41, L=12.0, D=10.0),
            configs.explicit_wall_channel(seed=42, L=14.0, D=12.0)]
    systems, a_type, r0, v = configs.concat(reps)
    gb = md.MdSystem(p, systems, a_type, r0, v, precision="mixed", nbr_capacity=160)
    gb.step(40)
    rb, vb, _, _ = gb.state()
    gb.close()
    off = 0
    for s, at, rr, vv in reps:
        g1 = md.MdSystem(p, s, at, rr, vv, precision="mixed", nbr_capacity=160)
        g1.step(40)
        r1, v1, _, _ = g1.state()
        g1.close()
        n = s.n_part
        assert np.array_equal(r1, rb[off:off + n]) and np.array_equal(v1, vb[off:off + n])
        off += n
