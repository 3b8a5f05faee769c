"""GPU parity of the virial and pressure tensors (mfa_get_virial) against the oracle.

Each term group's virial W_ab (minus the strain derivative of its energy; pinned in the oracle by
finite differences, tests/test_oracle_physics.py) is compared on the same state: through the
per-routine drop-ins on the try deck, on a batch of benchmark replicas and on a charged brush
(real-space Coulomb, reciprocal sum, slab dipole), and through the fused mixed-precision step.
Tolerance per group, relative to the group's largest component: FP64 1e-10, mixed 1e-5."""
import numpy as np
import pytest

from mfa_brush_gb300 import configs, md

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "mixed": 1e-5}


def close(w, wo, tol, what):
    scale = max(np.abs(wo).max(), 1e-300)
    err = np.abs(np.asarray(w) - np.asarray(wo)).max() / scale
    assert err <= tol, (what, err, w, wo)


def dropin_virial(g, routines):
    g.zero_force()
    for r in routines:
        getattr(g, r)()
    return g.virial()


ROUTINES = {"fluid_fluid": "pair", "fluid_wall": "wall", "intra_molec": "fene", "bending": "bend",
            "orientation": "orientation"}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_virial_dropins_try(gpu, try_deck, oracle_mod, precision):
    """try/conf_old: pair (LJ + DPD with its own cut-off), walls, FENE, bending and orientation
    groups, each routine alone."""
    inp, p, s, a_type, r0, v, a = try_deck
    g = md.MdSystem(p, s, a_type, r0, v, a, precision=precision)
    o = oracle_mod.Oracle(p, s, a_type, r0, v, a)
    for routine, group in ROUTINES.items():
        w = dropin_virial(g, [routine])[0]
        o.zero_force()
        getattr(o, routine)()
        wo = o.virial()[group]
        assert np.abs(wo).max() > 0, routine
        close(w[group], wo, TOL[precision], routine)
        if group != "orientation":
            assert np.array_equal(w[group], w[group].T)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_virial_batched_replicas(gpu, oracle_mod, precision):
    """Four replicas of the benchmark set in one context: pair, wall and FENE groups per replica."""
    p = configs.wca_params(gamma=5.0, kT=1.0, dt=0.005)
    reps = configs.replicas(256, 2024, indices=[3, 77, 150, 201])
    systems, a_type, r0, v = configs.concat(reps)
    g = md.MdSystem(p, systems, a_type, r0, v, precision=precision)
    ws = {r: dropin_virial(g, [r]) for r in ("fluid_fluid", "fluid_wall", "intra_molec")}
    for k, (s, at, rr, vv) in enumerate(reps):
        o = oracle_mod.Oracle(p, s, at, rr, vv)
        for routine in ws:
            o.zero_force()
            getattr(o, routine)()
            close(ws[routine][k][ROUTINES[routine]], o.virial()[ROUTINES[routine]], TOL[precision],
                  (k, routine))
        o.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_virial_charged_brush(gpu, oracle_mod, precision):
    """Slab Ewald: real-space Coulomb in the pair group, the reciprocal-space sum and the slab
    dipole term."""
    inp = configs.wca_inputs(gamma=1.0, thermostat=0)
    inp.flags.system = 3
    inp.charge[1], inp.charge[2] = -1.0, 1.0
    inp.alpha_c, inp.n_kmax, inp.rc_coul = 0.81, 5, 3.0
    p, _ = md.derive(inp)
    s, a_type, r0, v = configs.brush_channel(10.0, 10.0, 0.08, 10, rho=0.5, seed=21)
    g = md.MdSystem(p, s, a_type, r0, v, precision=precision)
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    o.ewald_init()
    w = dropin_virial(g, ["fluid_fluid", "ewald_k", "dipolar_correction"])[0]
    o.zero_force()
    o.fluid_fluid()
    o.ewald_k()
    o.dipolar_correction()
    wo = o.virial()
    for group in ("pair", "kspace", "dipole"):
        close(w[group], wo[group], TOL[precision], group)


def test_kinetic_tensor_and_pressure(gpu, try_deck, oracle_mod):
    """FP64 drop-in step: the kinetic tensor of verlet_velocities and the pressure tensor
    (kinetic + virial) / (Lx Ly D)."""
    inp, p, s, a_type, r0, v, a = try_deck
    g = md.MdSystem(p, s, a_type, r0, v, a, precision="fp64")
    g.md_step()
    w = g.virial()[0]
    o = oracle_mod.Oracle(p, s, a_type, r0, v, a)
    o.step(1, 1, 0)
    close(w["kinetic"], o.kinetic_tensor(), 1e-8, "kinetic")
    L = list(s.boundary)
    assert w["volume"] == L[0] * L[1] * L[2]
    tot = sum(w[k] for k in ("pair", "fene", "bend", "bend_melt", "orientation", "wall", "kspace", "dipole"))
    assert np.allclose(w["total"], tot, rtol=1e-14, atol=0)
    assert np.allclose(w["pressure"], (w["kinetic"] + w["total"]) / w["volume"], rtol=1e-14, atol=0)
