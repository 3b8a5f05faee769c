"""Seeded synthetic brush-channel configurations (the reference generates its own with gen_brush.f90;
none of its published inputs match these workloads).

Particles are laid on a simple-cubic lattice filling the channel interior (z in [0.9, D-0.9]), with
spacing chosen from the target density, so that no two beads start closer than ~0.95 sigma and
the first steps need no force switch-on.  Brush chains are lattice self-avoiding walks grown from
anchor sites drawn uniformly at random on the first and last z layer (first half of the chains on
the bottom wall, second half on the top wall, heads = bead 1 of each chain), biased away from the
wall; free (melt) chains are grown the same way from random free sites; solvent beads take
uniformly random free sites until the total density is reached.  Velocities are Maxwell-Boltzmann
at kT (heads at rest).  Order of particles follows the reference: brush chains, then melt /
solvent chains, then particle-4 chains (init_system.f90:172-187).

Workloads (sizes from the project's benchmark definitions):
  * replicas(256, seed)  -- 256 uneven WCA+FENE+DPD channels, grafting density U[0.05,0.3],
    N U{10..100}, D U[10,40], L U[15,40], solvent to 0.8 (a replica whose brush alone would
    exceed 70 % of its beads is redrawn from the same stream);
  * small_channel()      -- a 20x20x20 channel with 40 chains of 30 beads per wall and solvent
    to 0.8, the plain-FP64 reference-scale case.
"""
import numpy as np

from . import abi, md

# lattice moves: 6 face neighbours (bond a), then 12 edge neighbours (bond sqrt(2) a < R0), the
# latter with a small weight so a walk only uses them to escape a dead end
_NEIGH = np.array([[0, 0, 1], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, -1]] +
                  [[dx, dy, dz] for dx in (-1, 0, 1) for dy in (-1, 0, 1) for dz in (-1, 0, 1)
                   if abs(dx) + abs(dy) + abs(dz) == 2], np.int64)
_NW = len(_NEIGH)
_EDGE_W = 1e-3


Z_LO = 0.9  # first/last lattice layer: the repulsive 9-3 wall force there is ~100 eps/sigma


def _lattice(L, D, n_sites_min, z_lo=Z_LO, a_max=1.0):
    """Lattice dims (nx, nz) and spacings covering [0,L)^2 x [z_lo, D-z_lo] with at least
    n_sites_min sites strictly between the two anchor layers (z index 0 and nz-1).  Both spacings
    are at most a_max: a walk's face-diagonal step (taken when the axis steps are blocked) is then
    a bond of at most sqrt(2) a_max, short of the FENE limit of 1.5 (at 1.49, spacing 1.05, the
    bond force is ~4000 and the first steps can tear the chain at dt = 0.005)."""
    a = min(a_max, (L * L * max(D - 2 * z_lo, 0.5) / max(n_sites_min, 1)) ** (1.0 / 3.0))
    for _ in range(400):
        nx = max(3, int(np.ceil(L / a)))
        nz = max(3, int(np.ceil((D - 2 * z_lo) / a)) + 1)
        if nx * nx * (nz - 2) >= n_sites_min:
            break
        a *= 0.99
    ax = L / nx
    az = (D - 2 * z_lo) / (nz - 1)
    return nx, nz, ax, az


def brush_channel(L, D, sigma_g, n_mon, rho=0.8, seed=0, n_mon_d=1, n_chain_d=None, kT=1.0,
                  solvent_type=3, melt_type=3, max_fill=0.97, z_lo=Z_LO, wall_spacing=0.0, wall_type=4,
                  a_max=1.0):
    """One replica: returns (abi.System, a_type[n], r0[n,3], v[n,3]).  Types are the reference's:
    1 head, 2 brush bead, 3 melt/solvent.  wall_spacing > 0 appends explicit wall beads (type
    wall_type, at rest) on a square lattice of that spacing at z = 0 and z = D, after the mobile
    particles as in the reference (init_system.f90:172-187; gen_wall.f90 uses two beads per
    lattice cell, this generator one).  a_max caps the lattice spacing (see _lattice); a
    chain-free replica may raise it."""
    rng = np.random.default_rng(seed)
    n_chain = 2 * int(round(sigma_g * L * L))
    n_brush = n_chain * n_mon
    n_total = int(round(rho * L * L * D))
    if n_chain_d is None:
        n_chain_d = max(0, (n_total - n_brush) // n_mon_d)
    n_melt = n_chain_d * n_mon_d
    n = n_brush + n_melt
    nx, nz, ax, az = _lattice(L, D, int(np.ceil((n - n_chain) / max_fill)), z_lo, a_max)
    occ = np.zeros((nx, nx, nz), bool)
    # the first and last layer hold the brush heads only; no other bead may enter them
    occ[:, :, 0] = True
    occ[:, :, nz - 1] = True
    sites = np.zeros((n, 3), np.int64)

    def regrow(pos, ci, k, w0, movable=False):
        """Serial self-avoiding regrowth of beads 1..k of chain ci (its old sites are freed).  A
        free chain (movable) whose start is walled in moves its start to another free site after
        every 20 failed attempts; a grafted chain keeps its anchor."""
        old = pos[ci, 1:k]
        occ[old[:, 0], old[:, 1], old[:, 2]] = False
        for attempt in range(200):
            if movable and attempt and attempt % 20 == 0:
                occ[tuple(pos[ci, 0])] = False
                free_idx = np.flatnonzero(~occ.ravel())
                pos[ci, 0] = np.unravel_index(rng.choice(free_idx), occ.shape)
                occ[tuple(pos[ci, 0])] = True
            placed = []
            cur = pos[ci, 0]
            ok = True
            for kk in range(1, k + 1):
                cand = cur[None, :] + _NEIGH
                cand[:, 0] %= nx
                cand[:, 1] %= nx
                inz = (cand[:, 2] >= 0) & (cand[:, 2] < nz)
                cz = np.clip(cand[:, 2], 0, nz - 1)
                w = np.where(inz & ~occ[cand[:, 0], cand[:, 1], cz], w0, 0.0)
                if w.sum() <= 0:
                    ok = False
                    break
                j = rng.choice(_NW, p=w / w.sum())
                cur = cand[j]
                occ[tuple(cur)] = True
                placed.append(cur)
                pos[ci, kk] = cur
            if ok:
                return
            for p_ in placed:
                occ[tuple(p_)] = False
        raise RuntimeError("lattice walk stuck; lower the density or grafting density")

    def grow(starts, length, zdir):
        """Grows len(starts) lattice SAWs of `length` beads in parallel; returns [c, length, 3]."""
        c = len(starts)
        pos = np.zeros((c, length, 3), np.int64)
        pos[:, 0] = starts
        occ[starts[:, 0], starts[:, 1], starts[:, 2]] = True
        if zdir is not None:
            up = zdir[:, None] * _NEIGH[None, :, 2]
            wdir = np.where(up > 0, 3.0, np.where(up < 0, 0.3, 1.0))
        else:
            wdir = np.ones((c, _NW))
        wdir = wdir * np.where(np.abs(_NEIGH).sum(1) == 1, 1.0, _EDGE_W)[None, :]
        for k in range(1, length):
            cur = pos[:, k - 1]
            cand = cur[:, None, :] + _NEIGH[None, :, :]
            cand[:, :, 0] %= nx
            cand[:, :, 1] %= nx
            inz = (cand[:, :, 2] >= 0) & (cand[:, :, 2] < nz)
            cz = np.clip(cand[:, :, 2], 0, nz - 1)
            todo = np.arange(c)
            for _ in range(64):  # all chains claim at once; a site wanted twice goes to one of them
                free = inz[todo] & ~occ[cand[todo, :, 0], cand[todo, :, 1], cz[todo]]
                w = np.where(free, wdir[todo], 0.0)
                cw = np.cumsum(w, axis=1)
                stuck = cw[:, -1] <= 0
                if np.any(stuck):
                    # a walk trapped itself: regrow that chain alone (beads 1..k) from its anchor
                    for ci in todo[stuck]:
                        regrow(pos, ci, k, wdir[ci], movable=zdir is None)
                    todo = todo[~stuck]
                    if len(todo) == 0:
                        break
                    continue
                j = np.argmax(cw >= rng.random(len(todo))[:, None] * cw[:, -1:], axis=1)
                tgt = cand[todo, j]
                flat = (tgt[:, 0] * nx + tgt[:, 1]) * nz + tgt[:, 2]
                _, first = np.unique(flat, return_index=True)
                win = np.zeros(len(todo), bool)
                win[first] = True
                pos[todo[win], k] = tgt[win]
                occ[tgt[win, 0], tgt[win, 1], tgt[win, 2]] = True
                todo = todo[~win]
                if len(todo) == 0:
                    break
            if len(todo):
                raise RuntimeError("lattice walk could not resolve site conflicts")
        return pos

    # brush anchors: random distinct sites on the bottom (z=0) and top (z=nz-1) layers
    half = n_chain // 2
    cells = rng.choice(nx * nx, size=half, replace=False)
    cells_t = rng.choice(nx * nx, size=n_chain - half, replace=False)
    starts = np.concatenate([
        np.stack([cells // nx, cells % nx, np.zeros(half, np.int64)], 1),
        np.stack([cells_t // nx, cells_t % nx, np.full(n_chain - half, nz - 1, np.int64)], 1)])
    zdir = np.concatenate([np.ones(half), -np.ones(n_chain - half)])
    k = 0
    if n_chain:
        pos = grow(starts, n_mon, zdir)
        sites[:n_brush] = pos.reshape(-1, 3)
        k = n_brush
    if n_melt:
        free_idx = np.flatnonzero(~occ.ravel())
        pick = rng.choice(free_idx, size=n_chain_d, replace=False)
        st = np.stack(np.unravel_index(pick, occ.shape), 1).astype(np.int64)
        if n_mon_d == 1:
            occ[st[:, 0], st[:, 1], st[:, 2]] = True
            sites[k:k + n_melt] = st
        else:
            sites[k:k + n_melt] = grow(st, n_mon_d, None).reshape(-1, 3)
    r0 = np.empty((n, 3))
    r0[:, 0] = (sites[:, 0] + 0.5) * ax
    r0[:, 1] = (sites[:, 1] + 0.5) * ax
    r0[:, 2] = z_lo + sites[:, 2] * az
    a_type = np.full(n, solvent_type if n_mon_d == 1 else melt_type, np.int32)
    if n_chain:
        a_type[:n_brush] = 2
        a_type[0:n_brush:n_mon] = 1
    v = rng.normal(0.0, np.sqrt(kT), size=(n, 3))
    if n_chain:
        v[0:n_brush:n_mon] = 0.0
    n_mob = n
    if wall_spacing > 0:
        m = max(1, int(round(L / wall_spacing)))
        g = np.arange(m) * (L / m)
        gx, gy = np.meshgrid(g, g, indexing="ij")
        layer = np.stack([gx.ravel(), gy.ravel(), np.zeros(m * m)], 1)
        top = layer.copy()
        top[:, 2] = D
        r0 = np.concatenate([r0, layer, top])
        a_type = np.concatenate([a_type, np.full(2 * m * m, wall_type, np.int32)])
        v = np.concatenate([v, np.zeros((2 * m * m, 3))])
        n = len(r0)
    s = abi.System()
    s.boundary[0] = s.boundary[1] = L
    s.boundary[2] = D
    s.n_mon, s.n_chain = n_mon, n_chain
    s.n_mon_d, s.n_chain_d = n_mon_d, n_chain_d
    s.n_mon_e = s.n_chain_e = 0
    s.n_mon_tot = n_mob
    s.n_part = n
    s.s_time = 1
    s.seed = int(rng.integers(1, 2**63 - 1))
    return s, a_type, r0, v


def wca_inputs(gamma=5.0, kT=1.0, dt=0.005, a_w=-3.2, sigma_w=1.0, k_chain=30.0, r_chain=1.5,
               bending=False, k_bend=0.0, thermostat=0, wall=2, dpd_cut_off=0.0):
    """abi.Inputs of the WCA + FENE + DPD brush model expressed with the reference's own switches:
    SYSTEM 0, WALL 2 (repulsive 9-3 walls, A_w < 0) or WALL 1 (explicit wall beads, type 4),
    SOLVENT 1 (every pair cut at 2^(1/6) sigma), DPD inside the LJ cut-off (dpd_cut_off 0) or with
    its own cut-off (DPD_CUT_OFF), gamma = friction(1)."""
    inp = abi.Inputs()
    f = inp.flags
    f.system, f.symmetry, f.wall, f.solvent = 0, 0, wall, 1
    f.thermostat, f.dpd_weight, f.dpd_cut_off = thermostat, 0, dpd_cut_off
    f.bending = 1 if bending else 0
    f.bin_type, f.l_box = 2, 1
    inp.dt, inp.temp = dt, kT
    inp.x_space = inp.y_space = 1.0
    inp.n_cell_w_x = inp.n_cell_w_y = 1
    inp.z_space_wall = 1.0
    for t in range(4):
        inp.mass_type[t] = 1.0
        inp.sigma_ii[t] = 1.0
        inp.friction[t] = gamma
        for u in range(4):
            inp.epsil[t * abi.MAXT + u] = 1.0
    inp.a_w, inp.sigma_w = a_w, sigma_w
    inp.k_chain, inp.r_chain = k_chain, r_chain
    inp.k_bend = k_bend
    inp.hist_dim = 200
    return inp


def wca_params(**kw):
    p, _ = md.derive(wca_inputs(**kw))
    return p


def draw_replica_shapes(n_rep, seed, rho=0.8, max_brush_frac=0.7):
    """(sigma_g, N, D, L) per replica drawn from the seed."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n_rep:
        sg = rng.uniform(0.05, 0.3)
        N = int(rng.integers(10, 101))
        D = rng.uniform(10.0, 40.0)
        L = rng.uniform(15.0, 40.0)
        if 2 * sg * N > max_brush_frac * rho * D:
            continue
        out.append((sg, N, D, L))
    return out


def replicas(n_rep=256, seed=2024, rho=0.8, shapes=None, indices=None):
    """The batched workload: list of (System, a_type, r0, v), one per replica.  A lattice walk
    that traps itself is regrown from the next sub-seed (deterministic for a given seed).
    `indices` builds only those replicas of the set (each seeded by its index in the set)."""
    shapes = shapes or draw_replica_shapes(n_rep, seed, rho)
    reps = []
    for k in (range(len(shapes)) if indices is None else indices):
        sg, N, D, L = shapes[k]
        for attempt in range(50):
            try:
                reps.append(brush_channel(L, D, sg, N, rho=rho, seed=(seed * 100003 + k) * 64 + attempt))
                break
            except RuntimeError:
                continue
        else:
            raise RuntimeError("replica %d (%s) could not be generated" % (k, (sg, N, D, L)))
    return reps


def concat(reps):
    """Concatenates replicas into the batched host arrays of mfa_batch_init."""
    systems = [r[0] for r in reps]
    a_type = np.concatenate([r[1] for r in reps]).astype(np.int32)
    r0 = np.concatenate([r[2] for r in reps])
    v = np.concatenate([r[3] for r in reps])
    return systems, a_type, r0, v


def explicit_wall_channel(seed=1, L=20.0, D=20.0):
    """The plain-FP64 reference-scale case: L x L x D channel with explicit wall beads on a 1 sigma
    square lattice at z = 0 and z = D, grafting density 0.1 per wall (40 chains of 30 beads per
    wall at L = 20), solvent to total density 0.8; bead layers start 1 sigma from the walls.
    Use with wca_params(wall=1, dpd_cut_off=1.0)."""
    return brush_channel(L, D, 0.1, 30, rho=0.8, seed=seed, z_lo=1.0, wall_spacing=1.0)


def two_liquid_channel(L=20.0, D=16.0, sigma_g=0.15, n_mon=12, rho=0.8, seed=1):
    """Brush channel whose free liquid is split into layered halves: liquid A (type 3, melt
    chains of one bead) below D/2 and liquid B (type 4, particle-4 chains of one bead) above,
    ordered brush, A, B as the reference orders its molecules (init_system.f90:172-187).
    Use with two_liquid_inputs()."""
    s, a_type, r0, v = brush_channel(L, D, sigma_g, n_mon, rho=rho, seed=seed)
    n_brush = s.n_mon * s.n_chain
    free = np.arange(n_brush, s.n_mon_tot)
    a_idx = free[r0[free, 2] < D / 2]
    b_idx = free[r0[free, 2] >= D / 2]
    order = np.concatenate([np.arange(n_brush), a_idx, b_idx])
    a_type, r0, v = a_type[order].copy(), r0[order].copy(), v[order].copy()
    a_type[n_brush + len(a_idx):] = 4
    s.n_mon_d, s.n_chain_d = 1, len(a_idx)
    s.n_mon_e, s.n_chain_e = 1, len(b_idx)
    return s, a_type, r0, v


def two_liquid_inputs(gamma=5.0, kT=1.0, dt=0.005, eps_ab=0.5, f_x=0.01):
    """abi.Inputs of the two-liquid Poiseuille channel in the reference's switches: PARTICLE_4
    (liquid B), SOLVENT 3 with INTER4 4 (every pair cut at 2 * 2^(1/6) sigma), the brush in good
    solvent (WCA among brush beads), eps_AB between the liquids, WALL 2, POISEUILLE with the body
    force f_x, DPD in the LJ range, z-profiles on."""
    inp = wca_inputs(gamma=gamma, kT=kT, dt=dt)
    f = inp.flags
    f.solvent, f.particle_4, f.brush_in_good_sv = 3, 1, 1
    f.poiseuille, f.profiles = 1, 1
    inp.inter4 = 4
    # SOLVENT >= 2 takes the brush-liquid and A-B sigmas from system_input (non-additive)
    inp.delta_sig[0] = inp.delta_sig[1] = inp.delta_sig[2] = 1.0
    inp.a_w4, inp.sigma_w4 = inp.a_w, inp.sigma_w
    inp.epsil[2 * abi.MAXT + 3] = inp.epsil[3 * abi.MAXT + 2] = eps_ab
    inp.const_force[0] = f_x
    return inp


def charged_brush(gamma=5.0, seed=41):
    """The charged-brush channel at full size: 40 x 40 x 30, grafting density 0.1, N = 40, total
    density 0.7; slab Ewald (SYSTEM 3) with alpha_c = 0.81, real-space cut-off 3 and
    |k| <= 12 (2 pi / L) (8070 k-vectors under the reference's k-set rule), dipolar correction.
    Charge is per type in the reference, so "every 10th bead -1" (four charges per 40-bead chain)
    is spread over the 39 non-head beads of each chain (q = -4/39).  The same number of +1
    counterions (1280) are the fourth species (PARTICLE_4, single beads, WCA with everything),
    drawn at random among the free beads and stored after the neutral solvent, as the reference
    orders its molecules.  The lattice is filled to 75 % (at 97 %, on the wider lattice spacing
    that preceded the 1 sigma cap, this seed started with a contact that the FP64 reference
    algorithm did not survive).
    Returns (mfa_params, (System, a_type, r0, v))."""
    s, a_type, r0, v = brush_channel(40.0, 30.0, 0.1, 40, rho=0.7, seed=seed, max_fill=0.75)
    n_brush = s.n_mon * s.n_chain
    n_ci = 4 * s.n_chain
    rng = np.random.default_rng(seed + 1)
    free = np.arange(n_brush, s.n_mon_tot)
    ci = np.sort(rng.choice(free, n_ci, replace=False))
    solv = np.setdiff1d(free, ci)
    order = np.concatenate([np.arange(n_brush), solv, ci])
    a_type, r0, v = a_type[order].copy(), r0[order].copy(), v[order].copy()
    a_type[n_brush + len(solv):] = 4
    s.n_mon_d, s.n_chain_d = 1, len(solv)
    s.n_mon_e, s.n_chain_e = 1, n_ci
    inp = wca_inputs(gamma=gamma, thermostat=0)
    f = inp.flags
    f.system, f.particle_4 = 3, 1
    inp.inter4 = 1
    inp.a_w4, inp.sigma_w4 = inp.a_w, inp.sigma_w
    inp.charge[1] = -4.0 / (s.n_mon - 1)
    inp.charge[2] = 0.0
    inp.charge[3] = 1.0
    inp.alpha_c, inp.n_kmax, inp.rc_coul = 0.81, 12, 3.0
    p, _ = md.derive(inp)
    return p, (s, a_type, r0, v)


def melt_brush_inputs(gamma=5.0, kT=1.0, dt=0.005, eps_bm=1.2, k_bend=2.0):
    """abi.Inputs of the melt-in-brush model in the reference's switches: SOLVENT 3 (pairs cut at
    2 * 2^(1/6) sigma, the reference's nearest cut-off to 2.5 sigma) with BRUSH_IN_GOOD_SV
    (brush-brush WCA), eps = eps_bm between brush (heads included) and melt, eps = 1 otherwise,
    cosine bending (BENDING and BENDING_MELT, bend_form 1) with k_b on every chain, DPD inside
    each pair's LJ range, WALL 2.  The reference has no switch for a WCA melt next to an
    attractive brush-melt pair, so the melt-melt pairs share the 2 * 2^(1/6) sigma range."""
    inp = wca_inputs(gamma=gamma, kT=kT, dt=dt, bending=True, k_bend=k_bend)
    f = inp.flags
    f.solvent, f.brush_in_good_sv = 3, 1
    f.bending, f.bending_melt, f.orientation = 1, 1, 0
    inp.bend_form = 1
    inp.delta_sig[0] = 1.0  # SOLVENT >= 2 takes the brush-liquid sigma from system_input
    for b in (0, 1):
        inp.epsil[b * abi.MAXT + 2] = inp.epsil[2 * abi.MAXT + b] = eps_bm
    return inp


def melt_brush(L=100.0, D=40.0, sigma_g=0.2, n_mon=50, n_mon_d=20, rho=0.85, seed=5, **kw):
    """The large melt-in-brush channel: L x L x D, grafting density sigma_g per wall, brush chains
    of n_mon beads, free melt chains of n_mon_d beads to total density rho (340,000 particles at
    the defaults), lattice filled to 75 %.  Returns (mfa_params, (System, a_type, r0, v))."""
    s, a_type, r0, v = brush_channel(L, D, sigma_g, n_mon, rho=rho, n_mon_d=n_mon_d, seed=seed, max_fill=0.75)
    p, _ = md.derive(melt_brush_inputs(**kw))
    return p, (s, a_type, r0, v)


def two_liquid_large(seed=3):
    """The large two-liquid Poiseuille channel: 200 x 200 x 50, brushes at grafting density 0.15
    per wall with N = 30, liquids A and B in layered halves to total density 0.8 (1.6 M
    particles), eps_AB = 0.5, every liquid pair cut at 2 * 2^(1/6) sigma, body force f_x = 0.01,
    DPD gamma = 5, z-profiles on.  Returns (mfa_params, (System, a_type, r0, v))."""
    p, _ = md.derive(two_liquid_inputs(f_x=0.01))
    return p, two_liquid_channel(L=200.0, D=50.0, sigma_g=0.15, n_mon=30, rho=0.8, seed=seed)


def small_channel(seed=1):
    """20x20x20 channel, 40 chains of 30 beads per wall (grafting density 0.1), solvent to 0.8."""
    return brush_channel(20.0, 20.0, 0.1, 30, rho=0.8, seed=seed)
