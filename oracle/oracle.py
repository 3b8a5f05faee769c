"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the CPU FP64 oracle (oracle/libmfa_oracle.so).

Imported by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, and nowhere
else.  The oracle restates the reference's Fortran hot path in C (see mfa_oracle.c); it shares
only the plain data structs of include/mfa_gpu.h with the product.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libmfa_oracle.so")

_lib = None


def build(force=False):
    src = os.path.join(HERE, "mfa_oracle.c")
    hdr = os.path.join(os.path.dirname(HERE), "include", "mfa_gpu.h")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(src), os.path.getmtime(hdr)):
        subprocess.run(["make", "-s", "-C", HERE, "-B" if force else "all"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        from mfa_brush_gb300 import abi  # plain struct layouts only
        L = C.CDLL(LIB)
        P = C.POINTER
        vp, dp, ip = C.c_void_p, P(C.c_double), P(C.c_int32)
        sig = {
            "orc_derive_params": (C.c_int, [P(abi.Inputs), P(abi.Params), P(abi.System)]),
            "orc_force_switch_on": (None, [P(abi.Params), C.c_int64]),
            "orc_create": (vp, [P(abi.Params), P(abi.System), ip, dp, dp, dp]),
            "orc_destroy": (None, [vp]),
            "orc_make_cell_list": (C.c_int, [vp, C.c_int]),
            "orc_cell_info": (C.c_int, [vp, ip, ip, ip]),
            "orc_cell_neigh_list": (C.c_int, [ip, C.c_int32, ip]),
            "orc_fluid_fluid": (None, [vp]),
            "orc_fluid_fluid_omp": (None, [vp, C.c_int]),
            "orc_check_fluid_fluid": (C.c_double, [vp]),
            "orc_pair_list": (C.c_int64, [vp, ip, C.c_int64]),
            "orc_fluid_wall": (None, [vp]),
            "orc_wall_wall": (None, [vp]),
            "orc_intra_molec": (None, [vp]),
            "orc_bending": (None, [vp]),
            "orc_bending_melt": (None, [vp]),
            "orc_orientation": (None, [vp]),
            "orc_constant_force": (None, [vp]),
            "orc_ewald_init": (C.c_int, [vp]),
            "orc_ewald_kvecs": (C.c_int, [vp, dp, C.c_int]),
            "orc_ewald_k": (C.c_double, [vp]),
            "orc_dipolar_correction": (C.c_double, [vp]),
            "orc_verlet_positions": (None, [vp]),
            "orc_verlet_velocities": (None, [vp]),
            "orc_profiles_accumulate": (None, [vp]),
            "orc_get_profiles": (C.c_int64, [vp, dp, dp, dp]),
            "orc_forces": (None, [vp, C.c_int]),
            "orc_step": (None, [vp, C.c_int, C.c_int, C.c_int]),
            "orc_get_state": (None, [vp, dp, dp, dp, dp]),
            "orc_set_state": (None, [vp, dp, dp, dp]),
            "orc_set_force": (None, [vp, dp]),
            "orc_zero_force": (None, [vp]),
            "orc_set_step": (None, [vp, C.c_int64]),
            "orc_get_step": (C.c_int64, [vp]),
            "orc_set_r2min": (None, [vp, C.c_double]),
            "orc_get_energies": (None, [vp, dp]),
            "orc_observe": (None, [vp, dp]),
            "orc_pair_gauss": (C.c_double, [C.c_uint64, C.c_int64, C.c_int32, C.c_int32]),
            "orc_philox2x32": (None, [C.c_uint32, C.c_uint32, C.c_uint32, P(C.c_uint32)]),
            "orc_pair_key": (C.c_uint32, [C.c_uint64, C.c_int64]),
            "orc_track_force_scale": (None, [vp, C.c_int]),
            "orc_get_force_scale": (None, [vp, dp]),
            "orc_get_virial": (None, [vp, dp]),
            "orc_kinetic_tensor": (None, [vp, dp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _d(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int32))


VIRIAL_GROUPS = ("pair", "fene", "bend", "bend_melt", "orientation", "wall", "kspace", "dipole")

ENERGY_KEYS = ("v_fluid_fluid", "v_fluid_wall", "v_wall_wall", "v_intra_molec", "v_bend", "v_bend_melt",
               "v_or", "v_coul", "t_fluid")


def derive_params(inputs):
    from mfa_brush_gb300 import abi
    p, s = abi.Params(), abi.System()
    rc = lib().orc_derive_params(C.byref(inputs), C.byref(p), C.byref(s))
    assert rc == 0
    return p, s


class Oracle:
    """One replica held by the CPU restatement (FP64, the reference's loop order)."""

    def __init__(self, params, system, a_type, r0, v=None, a=None):
        self.L = lib()
        self.params, self.system = params, system
        self.n = system.n_part
        self.a_type = np.ascontiguousarray(a_type, np.int32)
        r0 = np.ascontiguousarray(r0, np.float64).reshape(self.n, 3)
        v = np.zeros_like(r0) if v is None else np.ascontiguousarray(v, np.float64).reshape(self.n, 3)
        a = np.zeros_like(r0) if a is None else np.ascontiguousarray(a, np.float64).reshape(self.n, 3)
        self.h = self.L.orc_create(C.byref(params), C.byref(system), _i(self.a_type), _d(r0), _d(v), _d(a))

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def state(self):
        r, v, a, f = (np.zeros((self.n, 3)) for _ in range(4))
        self.L.orc_get_state(self.h, _d(r), _d(v), _d(a), _d(f))
        return r, v, a, f

    def set_state(self, r0=None, v=None, a=None):
        c = lambda x: None if x is None else np.ascontiguousarray(x, np.float64).reshape(self.n, 3)
        self.L.orc_set_state(self.h, _d(c(r0)), _d(c(v)), _d(c(a)))

    def energies(self):
        e = np.zeros(9)
        self.L.orc_get_energies(self.h, _d(e))
        return dict(zip(ENERGY_KEYS, e))

    def __getattr__(self, name):
        # orc_<routine>(handle) pass-throughs: fluid_fluid, fluid_wall, intra_molec, ...
        f = getattr(lib(), "orc_" + name)
        return lambda *a: f(self.h, *a)

    def track_force_scale(self, on=True):
        """From the next force evaluation on, sum per particle the magnitudes of every force term
        acting on it (the conditioning of its force sum); serial pair loop."""
        self.L.orc_track_force_scale(self.h, 1 if on else 0)

    def force_scale(self):
        out = np.zeros(self.n)
        self.L.orc_get_force_scale(self.h, _d(out))
        return out

    def virial(self):
        """W_ab = sum of F_a r_b per term group of the last force evaluation (3x3 arrays)."""
        out = np.zeros(8 * 9)
        self.L.orc_get_virial(self.h, _d(out))
        return {g: out[9 * k:9 * k + 9].reshape(3, 3) for k, g in enumerate(VIRIAL_GROUPS)}

    def kinetic_tensor(self):
        out = np.zeros(9)
        self.L.orc_kinetic_tensor(self.h, _d(out))
        return out.reshape(3, 3)

    def observe(self):
        """observation.f90 quantities (see orc_observe)."""
        out = np.zeros(15)
        self.L.orc_observe(self.h, _d(out))
        return {"rg2_brush": out[0:3].tolist(), "rg2_melt": out[3:6].tolist(), "momentum": out[6:9].tolist(),
                "f_heads": [out[9:12].tolist(), out[12:15].tolist()]}

    def cell_info(self):
        nm = self.system.n_mon_tot
        cell_of = np.zeros(max(nm, 1), np.int32)
        nc = np.zeros(3, np.int32)
        nct = self.L.orc_cell_info(self.h, _i(cell_of), None, _i(nc))
        counts = np.zeros(nct + 1, np.int32)
        self.L.orc_cell_info(self.h, _i(cell_of), _i(counts), _i(nc))
        return cell_of[:nm], counts, nc

    def pair_list(self):
        n = self.L.orc_pair_list(self.h, None, 0)
        pairs = np.zeros((max(n, 1), 2), np.int32)
        self.L.orc_pair_list(self.h, _i(pairs), n)
        return pairs[:n]

    def kvecs(self):
        nk = self.L.orc_ewald_init(self.h)
        out = np.zeros((nk, 3))
        self.L.orc_ewald_kvecs(self.h, _d(out), nk)
        return out

    def profiles(self):
        H = self.params.hist_dim
        dens, vs, v2 = np.zeros((H, 3)), np.zeros((H, 3, 3)), np.zeros((H, 3, 3))
        n = self.L.orc_get_profiles(self.h, _d(dens), _d(vs), _d(v2))
        return dens, vs, v2, n


def cell_neigh_list(n_cells, n_nei):
    nc = np.ascontiguousarray(n_cells, np.int32)
    out = np.zeros(int(np.prod(nc)) * n_nei, np.int32)
    lib().orc_cell_neigh_list(_i(nc), n_nei, _i(out))
    return out.reshape(-1, n_nei)


def pair_gauss(seed, step, ta, tb):
    return lib().orc_pair_gauss(seed, step, ta, tb)
