"""Per-particle force gate on the exact kernels that the benchmark times.

One mfa_step(1) of the fused mixed-precision path (the pair kernel with the bonded terms fused
in, FP32 pair arithmetic, the integrator that adds the walls and the body force) produces the
forces that mfa_sync_to_host returns.  The oracle evaluates the forces of the same state: the
GPU's positions after that step, the half-kicked velocities that its pair kernel saw
(v(n+1) - dt/2 a(n+1), recomputed with the integrator's FP32 increment) and the same noise step,
with the DPD noise on.  Every mobile particle but the fixed brush heads is compared.

Gate: max_i |dF_i| / max(|F_i|, floor) <= 1e-5 with floor = FORCE_FLOOR_FRAC * F_rms: a particle
whose total force is far below the typical force is a near-cancelling sum of pair forces of
order F_rms, each evaluated in FP32 with a relative error of a few 1e-7, so its error is bounded
by the size of its terms, not by its total.  The fraction of particles whose plain relative
error |dF_i| / |F_i| is above 1e-5 is printed beside it."""
import numpy as np
import pytest

from mfa_brush_gb300 import configs, md

pytestmark = pytest.mark.gpu

FORCE_FLOOR_FRAC = 1e-2
GATE = 1e-5


def half_kick_velocities(p, vv, a):
    """v(n+1/2) = v(n+1) - dt/2 a(n+1) with the integrator's FP32 increment (the increment is
    formed in FP32 from the FP32 acceleration that the integrator stores)."""
    h = np.float32(0.5) * np.float32(p.dt)
    return vv - (h * a.astype(np.float32)).astype(np.float64)


def gate_stats(f, fo, floor_frac=FORCE_FLOOR_FRAC):
    nr = np.linalg.norm(fo, axis=1)
    rms = float(np.sqrt(np.mean(nr ** 2)))
    de = np.linalg.norm(f - fo, axis=1)
    gated = de / np.maximum(nr, floor_frac * rms)
    plain = de / np.maximum(nr, 1e-300)
    return {"gate_max": float(gated.max()), "frac_plain_over": float(np.mean(plain > GATE)),
            "max_over_rms": float(de.max() / rms), "n": int(len(nr)), "f_rms": rms,
            "floor_needed": float(np.max(de / GATE) / rms)}


def fused_forces_vs_oracle(oracle_mod, p, reps, warm=50, skin=0.5):
    """Runs `warm` fused mixed steps of the batch, then one more, and returns the (GPU, oracle)
    forces of every compared particle of every replica."""
    systems, a_type, r0, v = configs.concat(reps)
    g = md.MdSystem(p, systems, a_type, r0, v, precision="mixed", skin=skin)
    if warm:
        g.step(warm)
    g.step(1)
    r, vv, a, f = g.state()
    vh = half_kick_velocities(p, vv, a)
    out_g, out_o = [], []
    p0 = 0
    for s in systems:
        sl = slice(p0, p0 + s.n_part)
        o = oracle_mod.Oracle(p, s, a_type[sl], r[sl], vh[sl], a[sl])
        o.set_step(s.s_time + warm)
        o.forces(1)
        fo = o.state()[3]
        o.close()
        m = np.arange(s.n_part) < s.n_mon_tot
        if s.n_mon > 0:
            heads = np.arange(s.n_part) < s.n_mon * s.n_chain
            heads &= (np.arange(s.n_part) % max(s.n_mon, 1)) == 0
            m &= ~heads
        out_g.append(f[sl][m])
        out_o.append(fo[m])
        p0 += s.n_part
    g.close()
    return np.concatenate(out_g), np.concatenate(out_o)


def check(name, f, fo):
    st = gate_stats(f, fo)
    print("%s: %d particles, F_rms %.3g, max|dF|/F_rms %.3e, max |dF_i|/max(|F_i|, %.0e F_rms) %.3e, "
          "plain relative error > 1e-5 for %.4f%% of particles (floor that would pass: %.2e F_rms)"
          % (name, st["n"], st["f_rms"], st["max_over_rms"], FORCE_FLOOR_FRAC, st["gate_max"],
             100 * st["frac_plain_over"], st["floor_needed"]))
    assert st["gate_max"] <= GATE, st


def test_force_gate_brush_replicas(gpu, oracle_mod):
    """Replicas 0, 37, 128 and 255 of the 256-replica benchmark set, batched (WCA + FENE + DPD;
    one cut-off for every type pair, so the uniform-screening form of the pair kernel runs)."""
    p = configs.wca_params(gamma=5.0, kT=1.0, dt=0.005)
    reps = configs.replicas(256, 2024, indices=[0, 37, 128, 255])
    f, fo = fused_forces_vs_oracle(oracle_mod, p, reps)
    check("brush replicas", f, fo)


def test_force_gate_melt_in_brush(gpu, oracle_mod):
    """A 20 x 20 slab of the melt-in-brush channel (cosine bending on every chain, eps_bm 1.2,
    per-type cut-offs)."""
    p, (s, a_type, r0, v) = configs.melt_brush(L=20.0, D=40.0)
    f, fo = fused_forces_vs_oracle(oracle_mod, p, [(s, a_type, r0, v)])
    check("melt in brush", f, fo)


def test_force_gate_two_liquid(gpu, oracle_mod):
    """The two-liquid Poiseuille channel (eps_AB 0.5, body force on every non-head bead)."""
    p, _ = md.derive(configs.two_liquid_inputs(f_x=0.01))
    s, a_type, r0, v = configs.two_liquid_channel(L=20.0, D=16.0, seed=5)
    f, fo = fused_forces_vs_oracle(oracle_mod, p, [(s, a_type, r0, v)])
    check("two liquids", f, fo)
