"""Per-particle force gate on the exact kernels that the benchmark times.

One mfa_step(1) of the fused mixed-precision path (the pair kernel with the bonded terms fused
in, FP32 pair arithmetic, the integrator that adds the walls and the body force) produces the
forces that mfa_sync_to_host returns.  The oracle evaluates the forces of the same state: the
GPU's positions after that step, the half-kicked velocities that its pair kernel saw
(v(n+1) - dt/2 a(n+1), recomputed with the integrator's FP32 increment) and the same noise step,
with the DPD noise on.  Every mobile particle but the fixed brush heads is compared.

Gate: max_i |dF_i| / max(|F_i|, KAPPA * S_i) <= 1e-5, where S_i is the sum of the magnitudes of
every force term acting on particle i (each pair's LJ, DPD random, DPD dissipative and Coulomb
parts, each bond, angle, wall and body-force term), summed by the oracle.  FP32 evaluates every
term with a relative error of a few 1e-7, so the error of a particle's force is of the order of
1e-7 S_i whatever its total: a particle whose terms nearly cancel (|F_i| << S_i) cannot meet a
relative 1e-5 on |F_i| in any FP32 arithmetic.  The floor KAPPA * S_i leaves every particle whose
total is at least a tenth of its terms' size under the plain relative gate, and bounds the others
by their conditioning.  Printed beside it: max |dF_i| / F_rms, the plain relative error's largest
value among particles with |F_i| >= KAPPA * S_i, and the fraction of all particles whose plain
relative error |dF_i| / |F_i| is above 1e-5."""
import numpy as np
import pytest

from mfa_brush_gb300 import configs, md

pytestmark = pytest.mark.gpu

KAPPA = 0.1
GATE = 1e-5


def half_kick_velocities(p, vv, a):
    """v(n+1/2) = v(n+1) - dt/2 a(n+1) with the integrator's FP32 increment (the increment is
    formed in FP32 from the FP32 acceleration that the integrator stores)."""
    h = np.float32(0.5) * np.float32(p.dt)
    return vv - (h * a.astype(np.float32)).astype(np.float64)


def gate_stats(f, fo, scale, kappa=KAPPA):
    nr = np.linalg.norm(fo, axis=1)
    rms = float(np.sqrt(np.mean(nr ** 2)))
    de = np.linalg.norm(f - fo, axis=1)
    gated = de / np.maximum(nr, kappa * scale)
    plain = de / np.maximum(nr, 1e-300)
    well = nr >= kappa * scale
    return {"gate_max": float(gated.max()), "frac_plain_over": float(np.mean(plain > GATE)),
            "plain_max_well": float(plain[well].max()) if well.any() else 0.0,
            "frac_cancelling": float(np.mean(~well)),
            "max_over_scale": float(np.max(de / np.maximum(scale, 1e-300))),
            "max_over_rms": float(de.max() / rms), "n": int(len(nr)), "f_rms": rms}


def fused_forces_vs_oracle(oracle_mod, p, reps, warm=50, skin=0.5, virial=None):
    """Runs `warm` fused mixed steps of the batch, then one more, and returns the GPU forces, the
    oracle's forces and force scales of every compared particle of every replica.  With a list
    `virial`, appends per replica (the GPU's virial record of that step, the oracle's virial
    groups on the same forces, the kinetic tensor of the GPU's velocities)."""
    systems, a_type, r0, v = configs.concat(reps)
    g = md.MdSystem(p, systems, a_type, r0, v, precision="mixed", skin=skin)
    if warm:
        g.step(warm)
    g.step(1)
    r, vv, a, f = g.state()
    vh = half_kick_velocities(p, vv, a)
    wg = g.virial() if virial is not None else None
    out_g, out_o, out_s = [], [], []
    p0 = 0
    for k, s in enumerate(systems):
        sl = slice(p0, p0 + s.n_part)
        o = oracle_mod.Oracle(p, s, a_type[sl], r[sl], vh[sl], a[sl])
        o.set_step(s.s_time + warm)
        o.track_force_scale(True)
        o.forces(1)
        fo = o.state()[3]
        sc = o.force_scale()
        if virial is not None:
            m_ = np.array([p.mass_type[t - 1] for t in a_type[sl][:s.n_mon_tot]])
            vm = vv[sl][:s.n_mon_tot]
            virial.append((wg[k], o.virial(), np.einsum("i,ia,ib->ab", m_, vm, vm)))
        o.close()
        idx = np.arange(s.n_part)
        m = idx < s.n_mon_tot
        if s.n_mon > 0:  # the fixed brush heads (their force is reported as zero)
            m &= ~((idx < s.n_mon * s.n_chain) & (idx % s.n_mon == 0))
        out_g.append(f[sl][m])
        out_o.append(fo[m])
        out_s.append(sc[m])
        p0 += s.n_part
    g.close()
    return np.concatenate(out_g), np.concatenate(out_o), np.concatenate(out_s)


def check_virial(virial, groups):
    """The fused step's virial record against the oracle's, per group and replica (mixed 1e-5 of
    the group's largest component), and its kinetic tensor against the velocities'."""
    for wg, wo, kin in virial:
        for grp in groups:
            scale = np.abs(wo[grp]).max()
            assert scale > 0, grp
            assert np.abs(wg[grp] - wo[grp]).max() <= 1e-5 * scale, (grp, wg[grp], wo[grp])
        assert np.abs(wg["kinetic"] - kin).max() <= 1e-5 * np.abs(kin).max()


def check(name, f, fo, scale):
    st = gate_stats(f, fo, scale)
    print("%s: %d particles, F_rms %.3g; max |dF_i|/max(|F_i|, %.1f S_i) %.3e; max |dF_i|/S_i %.3e; "
          "max |dF|/F_rms %.3e; plain relative error: max %.3e over the %.2f%% of particles with "
          "|F_i| >= %.1f S_i, above 1e-5 for %.4f%% of all particles"
          % (name, st["n"], st["f_rms"], KAPPA, st["gate_max"], st["max_over_scale"], st["max_over_rms"],
             st["plain_max_well"], 100 * (1 - st["frac_cancelling"]), KAPPA, 100 * st["frac_plain_over"]))
    assert st["gate_max"] <= GATE, st


def test_force_gate_brush_replicas(gpu, oracle_mod):
    """Replicas 0, 37, 128 and 255 of the 256-replica benchmark set, batched (WCA + FENE + DPD;
    one cut-off for every type pair, so the uniform-screening form of the pair kernel runs)."""
    p = configs.wca_params(gamma=5.0, kT=1.0, dt=0.005)
    reps = configs.replicas(256, 2024, indices=[0, 37, 128, 255])
    vir = []
    check("brush replicas", *fused_forces_vs_oracle(oracle_mod, p, reps, virial=vir))
    check_virial(vir, ("pair", "fene", "wall"))


def test_force_gate_melt_in_brush(gpu, oracle_mod):
    """A 20 x 20 slab of the melt-in-brush channel (cosine bending on every chain, eps_bm 1.2,
    per-type cut-offs)."""
    p, (s, a_type, r0, v) = configs.melt_brush(L=20.0, D=40.0)
    vir = []
    check("melt in brush", *fused_forces_vs_oracle(oracle_mod, p, [(s, a_type, r0, v)], virial=vir))
    check_virial(vir, ("pair", "fene", "bend", "bend_melt", "wall"))


def test_force_gate_two_liquid(gpu, oracle_mod):
    """The two-liquid Poiseuille channel (eps_AB 0.5, body force on every non-head bead)."""
    p, _ = md.derive(configs.two_liquid_inputs(f_x=0.01))
    s, a_type, r0, v = configs.two_liquid_channel(L=20.0, D=16.0, seed=5)
    vir = []
    check("two liquids", *fused_forces_vs_oracle(oracle_mod, p, [(s, a_type, r0, v)], virial=vir))
    check_virial(vir, ("pair", "fene", "wall"))
