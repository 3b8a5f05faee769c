"""Observation on the device against the oracle: the averages of observation.f90 (fort.40 energy
means, fort.42 Rg^2 means, fort.43 r_par_per2, the momentum, obser_out.f90's pressure-tensor mean)
and the energy series of verlet_velocities.f90:184-207 (fort.60/61), over 50 observed steps after a
10-step relaxation, every step observed (energy_every 1), the DPD noise on.

The oracle runs the same steps on the same noise stream and its quantities are averaged here.
Tolerances, relative to each quantity's scale: FP64 1e-8 (the trajectories agree to ~1e-9);
mixed precision 1e-4 (its trajectory parts from the FP64 one at the 1e-7 level per step)."""
import numpy as np
import pytest

from mfa_brush_gb300 import configs, md

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-8, "mixed": 1e-4}
GROUPS = ("pair", "fene", "bend", "bend_melt", "orientation", "wall", "kspace", "dipole")


def near(a, b, tol, what):
    a, b = np.asarray(a, float), np.asarray(b, float)
    scale = max(np.abs(b).max(), 1e-12)
    assert np.abs(a - b).max() <= tol * scale, (what, a, b)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_observation_averages_and_series(gpu, oracle_mod, precision):
    p = configs.wca_params(gamma=5.0)
    s, a_type, r0, v = configs.brush_channel(14.0, 12.0, 0.15, 16, n_mon_d=8, seed=17, max_fill=0.75)
    assert s.n_chain_d > 0 and s.n_mon_d == 8
    relax, n_obs = 10, 50
    g = md.MdSystem(p, s, a_type, r0, v, precision=precision, energy_every=1, observe=True,
                    profile_from_step=relax, series_capacity=64)
    g.step(relax)
    g.step(n_obs)
    av = g.averages()[0]
    series = g.energy_series()
    assert g.energy_series() == []  # everything was returned by the first call
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    L = list(s.boundary)
    V = L[0] * L[1] * L[2]
    rows, orc_e = [], []
    for k in range(relax + n_obs):
        o.step(1, 1, 0)
        e = o.energies()
        orc_e.append(e)
        if k < relax:
            continue
        vt = e["v_wall_wall"] + e["v_fluid_wall"] + e["v_fluid_fluid"] + e["v_intra_molec"]
        ob = o.observe()
        w = o.virial()
        P = (o.kinetic_tensor() + sum(w[gr] for gr in GROUPS)) / V
        rb, rm = np.array(ob["rg2_brush"]), np.array(ob["rg2_melt"])
        rows.append({"v_total": vt, "t_total": e["t_fluid"], "e_total": vt + e["t_fluid"],
                     "v_fluid": e["v_fluid_fluid"] + e["v_intra_molec"] + e["v_fluid_wall"],
                     "e_fluid": e["v_fluid_fluid"] + e["t_fluid"], "momentum": np.array(ob["momentum"]),
                     "rg2_brush": rb, "rg2_melt": rm, "rg2_mean": 0.5 * (rb + rm),
                     "r_par_per2": np.array([(rb[2] - 0.5 * (rb[0] + rb[1])) / rb.sum(),
                                             (rm[2] - 0.5 * (rm[0] + rm[1])) / rm.sum()]),
                     "pressure": P, "f_heads": np.array(ob["f_heads"])})
    tol = TOL[precision]
    assert av["count"] == n_obs
    for key in ("v_total", "t_total", "e_total", "v_fluid", "e_fluid", "rg2_brush", "rg2_melt", "rg2_mean",
                "r_par_per2", "pressure", "f_heads"):
        near(av[key], np.mean([r[key] for r in rows], axis=0), tol, key)
    near(av["v_total2"], np.mean([r["v_total"] ** 2 for r in rows]), tol, "v_total2")
    # the momentum is a sum of cancelling terms: compare it on the scale of the particles' own
    m_scale = np.sqrt(s.n_mon_tot) * np.sqrt(np.mean(np.sum(v ** 2, axis=1)))
    assert np.abs(av["momentum"] - np.mean([r["momentum"] for r in rows], axis=0)).max() <= tol * m_scale
    # the series: one record per step, in order, with the oracle's energies of that step
    assert len(series) == relax + n_obs
    for k, rec in enumerate(series):
        e, eo = rec[0], orc_e[k]
        assert e["step"] == s.s_time + k + 1
        for key in ("v_fluid_fluid", "v_intra_molec", "v_fluid_wall", "t_fluid"):
            near(e[key], eo[key], tol, (k, key))
