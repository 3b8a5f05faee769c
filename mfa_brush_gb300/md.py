"""Python mirror of mfa_brush's per-step interface over the CUDA library.

`MdSystem` exposes the reference's subroutine names (md_main.f90:85-185) -- verlet_positions,
fluid_fluid, fluid_wall, wall_wall, intra_molec, bending, bending_melt, orientation, ewald_k,
dipolar_correction, constant_force, verlet_velocities -- plus the fused `step(n)` that runs
whole steps on the device.  Every call goes through the C ABI of include/mfa_gpu.h; nothing here
computes physics.  `read_deck` reads a reference input directory (control_simulation.h,
system_input, mfa_input, conf_old) with the library's own parsers.
"""
import ctypes as C
import os

import numpy as np

from . import abi


def _lib():
    return abi.load_library()


def flags_from_header(path):
    f = abi.Flags()
    abi.check(_lib().mfa_flags_from_header(path.encode(), C.byref(f)))
    return f


def read_inputs(deck_dir, flags=None, header="control_simulation.h"):
    """init_system + init_params reading of a deck directory -> abi.Inputs."""
    inp = abi.Inputs()
    inp.flags = flags if flags is not None else flags_from_header(os.path.join(deck_dir, header))
    lib = _lib()
    abi.check(lib.mfa_read_system_input(os.path.join(deck_dir, "system_input").encode(), C.byref(inp)))
    abi.check(lib.mfa_read_mfa_input(os.path.join(deck_dir, "mfa_input").encode(), C.byref(inp)))
    return inp


def derive(inp):
    p, s = abi.Params(), abi.System()
    abi.check(_lib().mfa_derive_params(C.byref(inp), C.byref(p), C.byref(s)))
    return p, s


def read_conf_old(path, n_part):
    a_type = np.zeros(n_part, np.int32)
    r0 = np.zeros((n_part, 3))
    v = np.zeros((n_part, 3))
    a = np.zeros((n_part, 3))
    abi.check(_lib().mfa_read_conf_old(path.encode(), n_part, abi.iptr(a_type), abi.dptr(r0), abi.dptr(v),
                                       abi.dptr(a)))
    return a_type, r0, v, a


def write_conf_new(path, inp, a_type, r0, v, a):
    n = len(a_type)
    abi.check(_lib().mfa_write_conf_new(path.encode(), C.byref(inp), n, abi.iptr(np.ascontiguousarray(a_type, np.int32)),
                                        abi.dptr(np.ascontiguousarray(r0, np.float64)),
                                        abi.dptr(np.ascontiguousarray(v, np.float64)),
                                        abi.dptr(np.ascontiguousarray(a, np.float64))))


def read_deck(deck_dir, conf="conf_old"):
    """(inputs, params, system, a_type, r0, v, a) of a reference input directory."""
    inp = read_inputs(deck_dir)
    p, s = derive(inp)
    a_type, r0, v, a = read_conf_old(os.path.join(deck_dir, conf), s.n_part)
    return inp, p, s, a_type, r0, v, a


def options(precision="mixed", skin=0.3, energy_every=10, use_graphs=True, device=0, nbr_capacity=0,
            profile_from_step=0, block_size=0, kspace_plain_sums=False, observe=False, series_capacity=0,
            list_cells=0, pair_schedule=0, separate_integrator=False, list_cells_x=0):
    o = abi.Options()
    _lib().mfa_default_options(C.byref(o))
    o.precision = abi.PREC_MIXED if precision in ("mixed", abi.PREC_MIXED) else abi.PREC_FP64
    o.skin = skin
    o.energy_every = energy_every
    o.use_graphs = 1 if use_graphs else 0
    o.device = device
    o.nbr_capacity = nbr_capacity
    o.profile_from_step = profile_from_step
    o.block_size = block_size
    o.kspace_plain_sums = 1 if kspace_plain_sums else 0
    o.observe = 1 if observe else 0
    o.series_capacity = series_capacity
    o.list_cells = list_cells
    o.pair_schedule = pair_schedule
    o.separate_integrator = 1 if separate_integrator else 0
    o.list_cells_x = list_cells_x
    return o


class MdSystem:
    """One device context holding R >= 1 replicas that share a parameter set."""

    def __init__(self, params, systems, a_type, r0, v=None, a=None, **opt):
        if isinstance(systems, abi.System):
            systems = [systems]
        self.lib = _lib()
        self.params = params
        self.systems = list(systems)
        self.nrep = len(self.systems)
        self.n = int(sum(s.n_part for s in self.systems))
        self.a_type = np.ascontiguousarray(a_type, np.int32)
        r0 = np.ascontiguousarray(r0, np.float64).reshape(self.n, 3)
        v = None if v is None else np.ascontiguousarray(v, np.float64).reshape(self.n, 3)
        a = None if a is None else np.ascontiguousarray(a, np.float64).reshape(self.n, 3)
        self.opt = options(**opt)
        sysarr = (abi.System * self.nrep)(*self.systems)
        self.ctx = C.c_void_p()
        rc = self.lib.mfa_batch_init(C.byref(params), self.nrep, sysarr, abi.iptr(self.a_type), abi.dptr(r0),
                                     abi.dptr(v), abi.dptr(a), C.byref(self.opt), C.byref(self.ctx))
        if rc != abi.MFA_OK:
            msg = self.lib.mfa_last_error(self.ctx).decode() if self.ctx.value else ""
            if self.ctx.value:
                self.lib.mfa_destroy(self.ctx)
            self.ctx = C.c_void_p()
            raise abi.MfaError(rc, msg)

    # -- lifetime ---------------------------------------------------------------------------
    def close(self):
        if self.ctx is not None and self.ctx.value:
            self.lib.mfa_destroy(self.ctx)
        self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, rc):
        return abi.check(rc, self.ctx)

    def _rep_out(self):
        return np.zeros(self.nrep)

    # -- md_main routines ---------------------------------------------------------------------
    def verlet_positions(self):
        self._ck(self.lib.mfa_verlet_positions(self.ctx))

    def check_skin(self):
        r = abi.i32(0)
        self._ck(self.lib.mfa_check_skin(self.ctx, C.byref(r)))
        return bool(r.value)

    def zero_force(self):
        self._ck(self.lib.mfa_zero_force(self.ctx))

    def fluid_fluid(self):
        vff, vc = self._rep_out(), self._rep_out()
        self._ck(self.lib.mfa_fluid_fluid(self.ctx, abi.dptr(vff), abi.dptr(vc)))
        return vff, vc

    def fluid_wall(self, wall_type=2):
        e = self._rep_out()
        self._ck(self.lib.mfa_fluid_wall(self.ctx, wall_type, abi.dptr(e)))
        return e

    def wall_wall(self, wall_type=2):
        e = self._rep_out()
        self._ck(self.lib.mfa_wall_wall(self.ctx, wall_type, abi.dptr(e)))
        return e

    def intra_molec(self):
        e = self._rep_out()
        self._ck(self.lib.mfa_intra_molec(self.ctx, abi.dptr(e)))
        return e

    def bending(self, mode=1):
        e = self._rep_out()
        self._ck(self.lib.mfa_bending(self.ctx, mode, abi.dptr(e)))
        return e

    def bending_melt(self, mode=1):
        e = self._rep_out()
        self._ck(self.lib.mfa_bending_melt(self.ctx, mode, abi.dptr(e)))
        return e

    def orientation(self, mode=1):
        e = self._rep_out()
        self._ck(self.lib.mfa_orientation(self.ctx, mode, abi.dptr(e)))
        return e

    def ewald_k(self, mode=1):
        e = self._rep_out()
        self._ck(self.lib.mfa_ewald_k(self.ctx, mode, abi.dptr(e)))
        return e

    def dipolar_correction(self):
        e = self._rep_out()
        self._ck(self.lib.mfa_dipolar_correction(self.ctx, abi.dptr(e)))
        return e

    def constant_force(self, mode=1):
        self._ck(self.lib.mfa_constant_force(self.ctx, mode))

    def verlet_velocities(self):
        e = (abi.Energies * self.nrep)()
        self._ck(self.lib.mfa_verlet_velocities(self.ctx, e))
        return [x.as_dict() for x in e]

    def profiles_accumulate(self):
        self._ck(self.lib.mfa_profiles_accumulate(self.ctx))

    def md_step(self, profiles=False):
        """One md_main iteration through the per-routine drop-ins (md_main.f90:85-202)."""
        f = self.params.flags
        self.verlet_positions()
        self.zero_force()
        self.fluid_fluid()
        if f.wall != 1:
            self.fluid_wall(f.wall)
        self.wall_wall(f.wall)
        self.intra_molec()
        if f.bending:
            self.bending(1)
        if f.bending_melt:
            self.bending_melt(1)
        if f.orientation:
            self.orientation(1)
        if f.system in (2, 3):
            self.ewald_k(1)
            self.dipolar_correction()
        if f.poiseuille:
            self.constant_force(1)
        e = self.verlet_velocities()
        if profiles:
            self.profiles_accumulate()
        return e

    # -- fused path -------------------------------------------------------------------------
    def step(self, n=1):
        self._ck(self.lib.mfa_step(self.ctx, int(n)))

    def synchronize(self):
        self._ck(self.lib.mfa_synchronize(self.ctx))

    def energies(self):
        e = (abi.Energies * self.nrep)()
        self._ck(self.lib.mfa_get_energies(self.ctx, e))
        return [x.as_dict() for x in e]

    def options_in_use(self):
        """The context's options (abi.Options), list_cells resolved to the value in use."""
        o = abi.Options()
        self._ck(self.lib.mfa_get_options(self.ctx, C.byref(o)))
        return o

    def list_cells(self):
        """List-build cells per list cut-off in use (1, 2 or 3)."""
        return self.options_in_use().list_cells

    def list_stats(self):
        """(neighbour-list capacity, largest list count seen at the rebuilds so far)."""
        cap, mx = abi.i32(0), abi.i32(0)
        self._ck(self.lib.mfa_list_stats(self.ctx, C.byref(cap), C.byref(mx)))
        return cap.value, mx.value

    def kspace_info(self, rep=None):
        """(k-vectors, charged particles) of the reciprocal-space sum of replica `rep` (replica 0
        when None); (0, 0) when uncharged."""
        nk, nq = abi.i32(0), abi.i32(0)
        if rep is None:
            self._ck(self.lib.mfa_kspace_info(self.ctx, C.byref(nk), C.byref(nq)))
        else:
            self._ck(self.lib.mfa_kspace_info_replica(self.ctx, rep, C.byref(nk), C.byref(nq)))
        return nk.value, nq.value

    def averages(self):
        """Observation averages of every replica (options observe=True), a list of dicts."""
        o = (abi.Averages * self.nrep)()
        self._ck(self.lib.mfa_get_averages(self.ctx, o))
        return [x.as_dict() for x in o]

    def reset_averages(self):
        self._ck(self.lib.mfa_reset_averages(self.ctx))

    def energy_series(self, cap=100000):
        """Energy records stored since the last call (options series_capacity > 0): a list over
        records of lists over replicas of energy dicts."""
        out = (abi.Energies * (cap * self.nrep))()
        n = abi.i32(0)
        self._ck(self.lib.mfa_get_energy_series(self.ctx, out, cap, C.byref(n)))
        return [[out[k * self.nrep + r].as_dict() for r in range(self.nrep)] for k in range(n.value)]

    def virial(self):
        """Virial tensors per term group, kinetic and pressure tensors of every replica, from the
        last energy record (see mfa_get_virial); a list of dicts of 3x3 arrays."""
        o = (abi.Virial * self.nrep)()
        self._ck(self.lib.mfa_get_virial(self.ctx, o))
        return [x.as_dict() for x in o]

    def observe(self):
        """observation.f90 quantities of every replica: Rg^2 (brush, melt), momentum, head forces."""
        o = (abi.Observables * self.nrep)()
        self._ck(self.lib.mfa_observe(self.ctx, o))
        return [x.as_dict() for x in o]

    def state(self):
        r, v, a, f = (np.zeros((self.n, 3)) for _ in range(4))
        self._ck(self.lib.mfa_sync_to_host(self.ctx, abi.dptr(r), abi.dptr(v), abi.dptr(a), abi.dptr(f)))
        return r, v, a, f

    def set_state(self, r0=None, v=None, a=None):
        c = lambda x: None if x is None else np.ascontiguousarray(x, np.float64).reshape(self.n, 3)
        self._ck(self.lib.mfa_set_state(self.ctx, abi.dptr(c(r0)), abi.dptr(c(v)), abi.dptr(c(a))))

    def step_index(self):
        s = abi.i64(0)
        self._ck(self.lib.mfa_get_step(self.ctx, C.byref(s)))
        return s.value

    def profiles(self, rep=0):
        H = self.params.hist_dim if self.params.hist_dim > 0 else 200
        dens, vs, v2 = np.zeros((H, 3)), np.zeros((H, 3, 3)), np.zeros((H, 3, 3))
        n = abi.i64(0)
        self._ck(self.lib.mfa_get_profiles(self.ctx, rep, abi.dptr(dens), abi.dptr(vs), abi.dptr(v2), C.byref(n)))
        return dens, vs, v2, n.value

    def reset_profiles(self):
        self._ck(self.lib.mfa_reset_profiles(self.ctx))

    # -- parity exports -----------------------------------------------------------------------
    def cell_list(self, rep=0, l_box=1):
        s = self.systems[rep]
        cell_of = np.zeros(max(1, s.n_mon_tot), np.int32)
        nc = np.zeros(3, np.int32)
        rc = self.params.r_cut_max
        L = np.array(list(s.boundary))
        est = np.maximum(1, (L / (rc if l_box == 1 else rc / 2)).astype(int) + 1)
        cap = int(np.prod(est)) + 1
        counts = np.zeros(cap, np.int32)
        self._ck(self.lib.mfa_cell_list(self.ctx, rep, l_box, abi.iptr(cell_of), abi.iptr(counts), cap,
                                        abi.iptr(nc)))
        nct = int(np.prod(nc))
        return cell_of[: s.n_mon_tot], counts[: nct + 1], nc

    def pair_list(self, rep=0, cap=None):
        s = self.systems[rep]
        cap = cap or max(1024, 64 * s.n_mon_tot)
        pairs = np.zeros((cap, 2), np.int32)
        n = abi.i64(0)
        self._ck(self.lib.mfa_pair_list(self.ctx, rep, abi.iptr(pairs), cap, C.byref(n)))
        if n.value > cap:
            return self.pair_list(rep, n.value)
        return pairs[: n.value]

    # -- timing -----------------------------------------------------------------------------
    def event_record(self, slot):
        self._ck(self.lib.mfa_event_record(self.ctx, slot))

    def event_elapsed(self, a, b):
        ms = C.c_float(0)
        self._ck(self.lib.mfa_event_elapsed(self.ctx, a, b, C.byref(ms)))
        return ms.value

    def kernel_times(self, nsteps):
        ms = (C.c_float * abi.NKFAM)()
        cnt = (abi.i32 * abi.NKFAM)()
        self._ck(self.lib.mfa_kernel_times(self.ctx, nsteps, ms, cnt))
        return {self.lib.mfa_kernel_name(k).decode(): (ms[k], cnt[k]) for k in range(abi.NKFAM)}

    def replica_rebuild_counts(self):
        """Rebuilds of each replica since the context was made."""
        out = np.zeros(self.nrep, np.int64)
        self._ck(self.lib.mfa_replica_rebuild_counts(self.ctx, out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out

    def rebuild_count(self):
        n = abi.i64(0)
        self._ck(self.lib.mfa_rebuild_count(self.ctx, C.byref(n)))
        return n.value

    def launch_count(self):
        n = abi.i64(0)
        self._ck(self.lib.mfa_launch_count(self.ctx, C.byref(n)))
        return n.value


def cell_neigh_list(n_cells, n_nei):
    nc = np.ascontiguousarray(n_cells, np.int32)
    out = np.zeros(int(np.prod(nc)) * n_nei, np.int32)
    abi.check(_lib().mfa_cell_neigh_list(abi.iptr(nc), n_nei, abi.iptr(out)))
    return out.reshape(-1, n_nei)


def device_count():
    n = abi.i32(0)
    _lib().mfa_device_count(C.byref(n))
    return n.value
