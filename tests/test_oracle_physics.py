"""Analytic checks of the oracle (CPU): forces are minus the gradient of the energies it reports,
pair and bonded forces obey Newton's third law, the linked-cell traversal finds the same pairs as
an O(N^2) search, and the half-shell cell table matches the reference's rules."""
import numpy as np
import pytest

from mfa_brush_gb300 import configs


def small_system(oracle_mod, thermostat=1, bending=True, seed=3, L=8.0, D=8.0):
    inp = configs.wca_inputs(bending=bending, k_bend=2.0, thermostat=thermostat)
    inp.flags.orientation = 1
    from mfa_brush_gb300 import md
    p, _ = md.derive(inp)
    s, a_type, r0, v = configs.brush_channel(L, D, 0.15, 8, rho=0.7, seed=seed)
    # jitter off the lattice so angles and distances are generic
    rng = np.random.default_rng(seed)
    r0 = r0 + rng.normal(0, 0.05, r0.shape)
    return p, s, a_type, r0, v


def total_energy(o, which):
    o.zero_force()
    getattr(o, which)()
    e = o.energies()
    key = {"fluid_fluid": "v_fluid_fluid", "fluid_wall": "v_fluid_wall", "intra_molec": "v_intra_molec",
           "bending": "v_bend", "orientation": "v_or"}[which]
    return e[key], o.state()[3]


@pytest.mark.parametrize("which", ["fluid_fluid", "fluid_wall", "intra_molec", "bending", "orientation"])
def test_force_is_minus_gradient(oracle_mod, which):
    p, s, a_type, r0, v = small_system(oracle_mod)
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    e0, f = total_energy(o, which)
    rng = np.random.default_rng(1)
    idx = rng.choice(s.n_mon_tot, 12, replace=False)
    h = 1e-6
    for i in idx:
        for d in range(3):
            rp = r0.copy(); rp[i, d] += h
            rm = r0.copy(); rm[i, d] -= h
            o.set_state(rp); ep, _ = total_energy(o, which)
            o.set_state(rm); em, _ = total_energy(o, which)
            fd = -(ep - em) / (2 * h)
            assert abs(fd - f[i, d]) <= 1e-5 * max(1.0, abs(f[i, d])), (which, i, d, fd, f[i, d])
    o.set_state(r0)


@pytest.mark.parametrize("thermostat", [0, 1])
def test_pair_newton3(oracle_mod, thermostat):
    p, s, a_type, r0, v = small_system(oracle_mod, thermostat=thermostat)
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    o.zero_force()
    o.fluid_fluid()
    f = o.state()[3]
    assert np.abs(f.sum(0)).max() < 1e-9 * np.abs(f).sum()


def test_cell_list_finds_all_pairs(oracle_mod):
    """Every pair inside the cut-off is visited exactly once by the 13-cell traversal."""
    p, s, a_type, r0, v = small_system(oracle_mod, L=9.0, D=9.0)
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    o.zero_force()
    o.fluid_fluid()
    e_cell = o.energies()["v_fluid_fluid"]
    e_n2 = o.check_fluid_fluid()
    assert abs(e_cell - e_n2) <= 1e-12 * max(1.0, abs(e_n2))


@pytest.mark.parametrize("n_cells,n_nei", [((5, 4, 6), 13), ((7, 6, 8), 62)])
def test_half_shell_table(oracle_mod, n_cells, n_nei):
    """make_cell_list2: each unordered pair of neighbouring cells appears once (x,y periodic,
    z bounded with the phantom cell 0)."""
    t = oracle_mod.cell_neigh_list(n_cells, n_nei)
    nx, ny, nz = n_cells
    reach = 1 if n_nei == 13 else 2
    seen = set()
    for c in range(1, nx * ny * nz + 1):
        for j in t[c - 1]:
            if j == 0:
                continue
            key = (min(c, j), max(c, j))
            assert key not in seen
            seen.add(key)
    # expected: all distinct neighbour pairs within `reach` (periodic x,y)
    def coords(c):
        c -= 1
        return c % nx, (c // nx) % ny, c // (nx * ny)
    exp = set()
    for c in range(1, nx * ny * nz + 1):
        x, y, z = coords(c)
        for dx in range(-reach, reach + 1):
            for dy in range(-reach, reach + 1):
                for dz in range(-reach, reach + 1):
                    if (dx, dy, dz) == (0, 0, 0) or not 0 <= z + dz < nz:
                        continue
                    j = 1 + (x + dx) % nx + ((y + dy) % ny) * nx + (z + dz) * nx * ny
                    exp.add((min(c, j), max(c, j)))
    assert seen == exp


def test_dpd_thermostat_temperature(oracle_mod):
    """DPD drives a WCA channel to kT (statistical; the reference's own check is fort.60's T)."""
    from mfa_brush_gb300 import md
    inp = configs.wca_inputs(gamma=5.0, kT=1.0, dt=0.005)
    inp.flags.dpd_cut_off = 1.5  # own DPD cut-off (DPD_CUT_OFF): a stronger thermostat than WCA range
    p, _ = md.derive(inp)
    s, a_type, r0, v = configs.brush_channel(8.0, 10.0, 0.1, 6, rho=0.6, seed=5)
    v = v * 0.3  # start cold
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    o.step(1500, 1, 0)
    ts = []
    for _ in range(40):
        o.step(25, 1, 0)
        ts.append(o.energies()["t_fluid"])
    n_free = s.n_mon_tot - s.n_chain
    kT = 2 * np.mean(ts) / (3 * n_free)
    assert abs(kT - 1.0) < 0.06, kT


def test_explicit_walls_cell_traversal_matches_n2(oracle_mod):
    """WALL 1: wall beads are in the cell list (BIN_TYPE 0 semantics), so the cell traversal sums
    the same LJ energy as the O(N^2) check over every particle, walls included."""
    from mfa_brush_gb300 import configs
    p = configs.wca_params(gamma=5.0, wall=1, dpd_cut_off=1.0)
    s, a_type, r0, v = configs.explicit_wall_channel(seed=3, L=10.0, D=10.0)
    assert s.n_part > s.n_mon_tot
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    o.zero_force()
    o.fluid_fluid()
    e_cell, e_n2 = o.energies()["v_fluid_fluid"], o.check_fluid_fluid()
    assert abs(e_cell - e_n2) <= 1e-12 * max(1.0, abs(e_n2))


def strained(r0, s, a, b, eps):
    """Positions and box under the strain r_a -> r_a + eps r_b: for a == b the axis and its box
    length (or the channel width, walls included) are scaled by 1 + eps."""
    from mfa_brush_gb300 import abi
    r = np.array(r0, np.float64).copy()
    s2 = abi.System.from_buffer_copy(s)
    if a == b:
        r[:, a] *= 1.0 + eps
        s2.boundary[a] = s.boundary[a] * (1.0 + eps)
    else:
        r[:, a] += eps * r[:, b]
    return r, s2


@pytest.mark.parametrize("group,which,key", [("pair", "fluid_fluid", "v_fluid_fluid"),
                                             ("fene", "intra_molec", "v_intra_molec"),
                                             ("bend", "bending", "v_bend"),
                                             ("orientation", "orientation", "v_or"),
                                             ("wall", "fluid_wall", "v_fluid_wall")])
def test_virial_is_minus_the_strain_derivative(oracle_mod, group, which, key):
    """W_ab of each group is -dU/de under r_a -> r_a + e r_b (central differences): the diagonal
    with the box (or the channel width, walls included) scaled, and the x-z and y-z shears."""
    p, s, a_type, r0, v = small_system(oracle_mod)
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    o.zero_force()
    getattr(o, which)()
    W = o.virial()[group]
    h = 1e-6
    for a, b in ((0, 0), (1, 1), (2, 2), (0, 2), (1, 2)):
        E = []
        for e in (h, -h):
            r, s2 = strained(r0, s, a, b, e)
            o2 = oracle_mod.Oracle(p, s2, a_type, r, v)
            o2.zero_force()
            getattr(o2, which)()
            E.append(o2.energies()[key])
            o2.close()
        fd = -(E[0] - E[1]) / (2 * h)
        assert abs(fd - W[a, b]) <= 1e-5 * max(1.0, np.abs(W).max()), (group, a, b, fd, W[a, b])
    if group != "orientation":  # central or rotation-invariant terms: a symmetric tensor
        assert np.abs(W - W.T).max() <= 1e-9 * max(1.0, np.abs(W).max())


def test_ewald_virial_is_minus_the_strain_derivative(oracle_mod):
    """The same for the charged brush (slab Ewald): real-space Coulomb (pair group), the
    reciprocal sum and the slab dipole term, each a function of the box as well."""
    from mfa_brush_gb300 import md
    inp = configs.wca_inputs(gamma=1.0, thermostat=1)
    inp.flags.system = 3
    inp.charge[1], inp.charge[2] = -1.0, 1.0
    inp.alpha_c, inp.n_kmax, inp.rc_coul = 0.81, 5, 3.0
    p, _ = md.derive(inp)
    s, a_type, r0, v = configs.brush_channel(10.0, 10.0, 0.08, 10, rho=0.5, seed=21)
    rng = np.random.default_rng(2)
    r0 = r0 + rng.normal(0, 0.05, r0.shape)
    # a rectangular box (y stretched by 3 %): in the square one several k-vectors sit exactly on
    # the |k| <= k_c boundary of the k-set rule, and a strain of 1e-6 moves them in or out
    r0[:, 1] *= 1.03
    s.boundary[1] *= 1.03

    def energies(sys_, r):
        o = oracle_mod.Oracle(p, sys_, a_type, r, v)
        nk = o.ewald_init()
        o.zero_force()
        o.fluid_fluid()
        e = o.energies()
        u_real = e["v_fluid_fluid"] + e["v_coul"]  # LJ and real-space Coulomb (self term: a constant)
        u_k = o.ewald_k()
        u_d = o.dipolar_correction()
        w = o.virial()
        o.close()
        return nk, {"pair": u_real, "kspace": u_k, "dipole": u_d}, w

    nk0, _, W = energies(s, r0)
    h = 1e-6
    for a, b in ((0, 0), (1, 1), (2, 2), (0, 2), (1, 2)):
        (nk1, ep, _), (nk2, em, _) = (energies(*strained(r0, s, a, b, e)[::-1]) for e in (h, -h))
        assert nk1 == nk2 == nk0
        # the reciprocal-space formula is the derivative under a deformation of the whole cell;
        # a shear of the positions alone in an orthorhombic box is not one, so the k-space term
        # is checked on the diagonal (box scalings) and for symmetry
        for g in (("pair", "kspace", "dipole") if a == b else ("pair", "dipole")):
            fd = -(ep[g] - em[g]) / (2 * h)
            assert abs(fd - W[g][a, b]) <= 1e-5 * max(1.0, np.abs(W[g]).max()), (g, a, b, fd, W[g][a, b])
    for g in ("pair", "kspace", "dipole"):
        assert np.abs(W[g] - W[g].T).max() <= 1e-9 * max(1.0, np.abs(W[g]).max())


def test_sheared_heads_and_refusals(oracle_mod):
    """The wall velocity of the brush-brush shear reaches the tables of both derivations; the
    oracle moves the heads at +-va_wall; a moving wall is refused with the body force
    (init_params.f90:899-907) and, with explicit walls, for a z velocity."""
    import numpy as np
    from mfa_brush_gb300 import abi, configs, md
    inp = configs.wca_inputs(gamma=5.0, kT=1.0, dt=0.005)
    inp.va_spring_twall[0], inp.va_spring_twall[1] = 0.25, 0.5
    p, _ = md.derive(inp)
    po, _ = oracle_mod.derive_params(inp)
    assert tuple(p.va_wall) == tuple(po.va_wall) == (0.25, 0.5)
    s, a_type, r0, v = configs.brush_channel(12.0, 10.0, 0.15, 10, seed=3)
    o = oracle_mod.Oracle(po, s, a_type, r0, v)
    o.step(5, 1, 0)
    vv = o.state()[1]
    heads = np.arange(s.n_chain) * s.n_mon
    sg = np.where(np.arange(s.n_chain) < s.n_chain // 2, 1.0, -1.0)
    assert np.array_equal(vv[heads, 0], 0.25 * sg) and np.array_equal(vv[heads, 1], 0.5 * sg)
    o.close()
    for flag in ("poiseuille", "wall1_z"):
        bad = configs.wca_inputs(gamma=5.0, wall=1 if flag == "wall1_z" else 2)
        bad.va_spring_twall[0] = 0.1
        if flag == "poiseuille":
            bad.flags.poiseuille = 1
        else:
            bad.va_spring_twall[2] = 0.1
        with pytest.raises(abi.MfaError):
            md.derive(bad)


def test_moving_explicit_walls_oracle(oracle_mod):
    """WALL 1 with a wall velocity (verlet_positions.f90:214-247): after n steps the oracle's
    wall beads 1..n_wall/2 sit at x0 + n va dt and the others at x0 - n va dt (wrapped), z
    unchanged; the heads move at +-va_wall."""
    import numpy as np
    from mfa_brush_gb300 import configs, md
    inp = configs.wca_inputs(gamma=5.0, wall=1, dpd_cut_off=1.0)
    inp.va_spring_twall[0], inp.va_spring_twall[1] = 0.5, -0.25
    p, _ = md.derive(inp)
    po, _ = oracle_mod.derive_params(inp)
    assert tuple(po.va_wall) == (0.5, -0.25)
    s, a_type, r0, v = configs.explicit_wall_channel(seed=3)
    o = oracle_mod.Oracle(po, s, a_type, r0, v)
    n = 7
    o.step(n, 1, 0)
    r, vv = o.state()[:2]
    o.close()
    nm, nw = s.n_mon_tot, s.n_part - s.n_mon_tot
    L = np.array(list(s.boundary))
    sg = np.where(np.arange(nw) < nw // 2, 1.0, -1.0)
    for d, va in ((0, 0.5), (1, -0.25)):
        x = r0[nm:, d].copy()
        for _ in range(n):  # the same additions and wraps as the position update
            x = np.where(sg > 0, x + va * po.dt, x - va * po.dt)
            x = np.where(x > L[d], x - L[d], np.where(x < 0.0, x + L[d], x))
        assert np.array_equal(r[nm:, d], x)
    assert np.array_equal(r[nm:, 2], r0[nm:, 2])
    assert np.all(vv[nm:] == 0.0)
    heads = np.arange(s.n_chain) * s.n_mon
    hs = np.where(np.arange(s.n_chain) < s.n_chain // 2, 1.0, -1.0)
    assert np.array_equal(vv[heads, 0], 0.5 * hs) and np.array_equal(vv[heads, 1], -0.25 * hs)
