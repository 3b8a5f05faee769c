"""ctypes view of include/mfa_gpu.h and the loader of the in-tree CUDA library.

The library (mfa_brush_gb300/libmfa_gb300.so) is the product; this module only describes its C
ABI to Python.  Loading fails loudly when the library is missing: there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmfa_gb300.so")
MAXT = 6

MFA_OK = 0
ERRORS = {
    -1: "MFA_ERR_ARG", -2: "MFA_ERR_CUDA", -3: "MFA_ERR_ALLOC", -4: "MFA_ERR_NLIST_OVERFLOW",
    -5: "MFA_ERR_OUT_OF_BOX", -6: "MFA_ERR_NAN", -7: "MFA_ERR_IO", -8: "MFA_ERR_PARSE",
    -9: "MFA_ERR_UNSUPPORTED", -10: "MFA_ERR_NO_DEVICE", -11: "MFA_ERR_STATE", -12: "MFA_ERR_CAPACITY",
}
PREC_FP64 = 0
PREC_MIXED = 1
COMPAT_EWALD_INV_PI = 1
COMPAT_EWALD_I_ONLY = 2
COMPAT_COUL_IN_LJ = 4

i32, i64, u32, u64, f64 = C.c_int32, C.c_int64, C.c_uint32, C.c_uint64, C.c_double


class Flags(C.Structure):
    _fields_ = [("system", i32), ("symmetry", i32), ("wall", i32), ("solvent", i32),
                ("hydrophobia", i32), ("brush_in_good_sv", i32), ("bending", i32),
                ("bending_melt", i32), ("orientation", i32), ("particle_4", i32),
                ("thermostat", i32), ("dpd_weight", i32), ("dpd_cut_off", f64),
                ("force_switch_on", i32), ("poiseuille", i32), ("profiles", i32),
                ("bin_type", i32), ("l_box", i32), ("free_heads", i32), ("sheared", i32)]


class Inputs(C.Structure):
    _fields_ = [("flags", Flags),
                ("n_mon", i32), ("n_chain", i32), ("n_cell_w_x", i32), ("n_cell_w_y", i32),
                ("n_mon_d", i32), ("n_chain_d", i32),
                ("drop_cell_x", f64), ("drop_cell_y", f64), ("z_skin", f64),
                ("n_mon_e", i32), ("n_chain_e", i32), ("inter4", i32),
                ("delta_sig", f64 * 3),
                ("a_w", f64), ("sigma_w", f64), ("a_w4", f64), ("sigma_w4", f64),
                ("charge", f64 * MAXT), ("alpha_c", f64), ("n_kmax", i32),
                ("const_force", f64 * 3),
                ("s_time", i64), ("n_relax", i64), ("n_obser", i64), ("n_safe", i64),
                ("dt", f64), ("temp", f64), ("x_space", f64), ("y_space", f64), ("z_space_wall", f64),
                ("mass_type", f64 * MAXT), ("epsil", f64 * (MAXT * MAXT)), ("sigma_ii", f64 * MAXT),
                ("friction", f64 * MAXT),
                ("k_spring_wall", f64), ("k_bend", f64), ("alpha_eq", f64),
                ("iseed", i64), ("k_chain", f64), ("r_chain", f64),
                ("f_twall", i32 * 3), ("va_spring_twall", f64 * 3), ("k_spring_twall", f64 * 3),
                ("bend_form", i32), ("rc_coul", f64), ("compat", u32), ("hist_dim", i32)]


T2 = f64 * (MAXT * MAXT)


class Params(C.Structure):
    _fields_ = [("flags", Flags), ("n_type", i32), ("dt", f64), ("temp", f64),
                ("mass_type", f64 * MAXT), ("epsil", T2), ("sigma", T2), ("sigma_2", T2),
                ("range_2", T2), ("inv_range_2", T2), ("e_shift", T2),
                ("r_cut_max", f64), ("r_cut_dpd_2", f64), ("friction1", f64), ("sig", f64),
                ("sigma_wall", f64 * MAXT), ("a_wall", f64 * MAXT), ("a_w", f64), ("sigma_w", f64),
                ("k_chain", f64), ("r_chain_2", f64), ("inv_r_chain_2", f64),
                ("k_bend", f64), ("alpha_eq", f64), ("k_or", f64), ("alpha_or", f64),
                ("bend_form", i32), ("const_force", f64 * 3), ("charge", f64 * MAXT),
                ("alpha_c", f64), ("sqrt_alpha", f64), ("inv_sqrt_pi", f64), ("n_kmax", i32),
                ("rc_coul_2", f64), ("skin", f64), ("r_2_min_init", f64), ("r_2_min_time", f64),
                ("compat", u32), ("hist_dim", i32), ("va_wall", f64 * 2)]

    def table(self, name):
        """n_type x n_type numpy copy of a row-major MAXT x MAXT table."""
        a = np.ctypeslib.as_array(getattr(self, name)).reshape(MAXT, MAXT)
        return a[: self.n_type, : self.n_type].copy()


class System(C.Structure):
    _fields_ = [("boundary", f64 * 3), ("n_mon", i32), ("n_chain", i32), ("n_mon_d", i32),
                ("n_chain_d", i32), ("n_mon_e", i32), ("n_chain_e", i32), ("n_mon_tot", i32),
                ("n_part", i32), ("s_time", i64), ("seed", u64)]


class Options(C.Structure):
    _fields_ = [("precision", i32), ("device", i32), ("skin", f64), ("nbr_capacity", i32),
                ("energy_every", i32), ("use_graphs", i32), ("block_size", i32),
                ("profile_from_step", i32), ("kspace_plain_sums", i32), ("observe", i32),
                ("series_capacity", i32), ("list_cells", i32), ("pair_schedule", i32),
                ("separate_integrator", i32), ("list_cells_x", i32)]


class Energies(C.Structure):
    _fields_ = [("step", i64), ("v_fluid_fluid", f64), ("v_fluid_wall", f64), ("v_wall_wall", f64),
                ("v_intra_molec", f64), ("v_bend", f64), ("v_bend_melt", f64), ("v_or", f64),
                ("v_coul", f64), ("t_fluid", f64), ("v_total", f64), ("e_total", f64), ("inv_n", f64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Observables(C.Structure):
    _fields_ = [("step", i64), ("rg2_brush", f64 * 3), ("rg2_melt", f64 * 3), ("momentum", f64 * 3),
                ("f_heads", (f64 * 3) * 2)]

    def as_dict(self):
        return {"step": self.step, "rg2_brush": list(self.rg2_brush), "rg2_melt": list(self.rg2_melt),
                "momentum": list(self.momentum), "f_heads": [list(self.f_heads[0]), list(self.f_heads[1])]}


class Averages(C.Structure):
    _fields_ = ([("count", i64)] +
                [(k, f64) for k in ("v_total", "t_total", "e_total", "v_total2", "t_total2", "e_total2",
                                    "v_fluid", "t_fluid", "e_fluid", "v_fluid2", "t_fluid2", "e_fluid2")] +
                [("momentum", f64 * 3), ("rg2_brush", f64 * 3), ("rg2_melt", f64 * 3), ("rg2_mean", f64 * 3),
                 ("r_par_per2", f64 * 2), ("pressure", f64 * 9), ("f_heads", (f64 * 3) * 2)])

    def as_dict(self):
        import numpy as np
        d = {}
        for k, t in self._fields_:
            x = getattr(self, k)
            d[k] = np.array(list(x)) if hasattr(x, "__len__") else x
        d["pressure"] = d["pressure"].reshape(3, 3)
        return d


VIRIAL_GROUPS = ("pair", "fene", "bend", "bend_melt", "orientation", "wall", "kspace", "dipole")


class Virial(C.Structure):
    _fields_ = ([("step", i64)] + [(g, f64 * 9) for g in VIRIAL_GROUPS] +
                [("total", f64 * 9), ("kinetic", f64 * 9), ("volume", f64), ("pressure", f64 * 9)])

    def as_dict(self):
        """3x3 arrays (row-major w[3 a + b] = sum of F_a r_b), plus step and volume."""
        import numpy as np
        d = {"step": self.step, "volume": self.volume}
        for k in VIRIAL_GROUPS + ("total", "kinetic", "pressure"):
            d[k] = np.array(list(getattr(self, k))).reshape(3, 3)
        return d


P = C.POINTER
vp = C.c_void_p
dp = P(f64)
ip = P(i32)

# name -> (restype, argtypes)
SIGNATURES = {
    "mfa_version": (C.c_char_p, []),
    "mfa_device_count": (i32, [ip]),
    "mfa_default_options": (None, [P(Options)]),
    "mfa_flags_from_header": (i32, [C.c_char_p, P(Flags)]),
    "mfa_read_system_input": (i32, [C.c_char_p, P(Inputs)]),
    "mfa_read_mfa_input": (i32, [C.c_char_p, P(Inputs)]),
    "mfa_derive_params": (i32, [P(Inputs), P(Params), P(System)]),
    "mfa_read_conf_old": (i32, [C.c_char_p, i32, ip, dp, dp, dp]),
    "mfa_write_conf_new": (i32, [C.c_char_p, P(Inputs), i32, ip, dp, dp, dp]),
    "mfa_force_switch_on": (i32, [P(Params), i64, i64]),
    "mfa_init": (i32, [P(Params), P(System), ip, dp, dp, dp, P(Options), P(vp)]),
    "mfa_batch_init": (i32, [P(Params), i32, P(System), ip, dp, dp, dp, P(Options), P(vp)]),
    "mfa_destroy": (i32, [vp]),
    "mfa_last_error": (C.c_char_p, [vp]),
    "mfa_synchronize": (i32, [vp]),
    "mfa_stream": (vp, [vp]),
    "mfa_n_particles": (i32, [vp, P(i64), ip]),
    "mfa_verlet_positions": (i32, [vp]),
    "mfa_check_skin": (i32, [vp, ip]),
    "mfa_zero_force": (i32, [vp]),
    "mfa_fluid_fluid": (i32, [vp, dp, dp]),
    "mfa_fluid_wall": (i32, [vp, i32, dp]),
    "mfa_wall_wall": (i32, [vp, i32, dp]),
    "mfa_intra_molec": (i32, [vp, dp]),
    "mfa_bending": (i32, [vp, i32, dp]),
    "mfa_bending_melt": (i32, [vp, i32, dp]),
    "mfa_orientation": (i32, [vp, i32, dp]),
    "mfa_ewald_k": (i32, [vp, i32, dp]),
    "mfa_dipolar_correction": (i32, [vp, dp]),
    "mfa_constant_force": (i32, [vp, i32]),
    "mfa_verlet_velocities": (i32, [vp, P(Energies)]),
    "mfa_profiles_accumulate": (i32, [vp]),
    "mfa_step": (i32, [vp, i32]),
    "mfa_get_step": (i32, [vp, P(i64)]),
    "mfa_sync_to_host": (i32, [vp, dp, dp, dp, dp]),
    "mfa_set_state": (i32, [vp, dp, dp, dp]),
    "mfa_get_energies": (i32, [vp, P(Energies)]),
    "mfa_get_profiles": (i32, [vp, i32, dp, dp, dp, P(i64)]),
    "mfa_observe": (i32, [vp, P(Observables)]),
    "mfa_get_virial": (i32, [vp, P(Virial)]),
    "mfa_get_averages": (i32, [vp, P(Averages)]),
    "mfa_reset_averages": (i32, [vp]),
    "mfa_get_energy_series": (i32, [vp, P(Energies), i32, ip]),
    "mfa_list_stats": (i32, [vp, ip, ip]),
    "mfa_get_options": (i32, [vp, P(Options)]),
    "mfa_kspace_info": (i32, [vp, ip, ip]),
    "mfa_kspace_info_replica": (i32, [vp, i32, ip, ip]),
    "mfa_reset_profiles": (i32, [vp]),
    "mfa_cell_list": (i32, [vp, i32, i32, ip, ip, i32, ip]),
    "mfa_cell_neigh_list": (i32, [ip, i32, ip]),
    "mfa_pair_list": (i32, [vp, i32, ip, i64, P(i64)]),
    "mfa_pair_list_static": (i32, [vp, i32, ip, i64, P(i64)]),
    "mfa_event_record": (i32, [vp, i32]),
    "mfa_event_elapsed": (i32, [vp, i32, i32, P(C.c_float)]),
    "mfa_kernel_times": (i32, [vp, i32, P(C.c_float), ip]),
    "mfa_kernel_name": (C.c_char_p, [i32]),
    "mfa_fp32_fma_peak": (i32, [i32, dp]),
    "mfa_launch_count": (i32, [vp, P(i64)]),
    "mfa_rebuild_count": (i32, [vp, P(i64)]),
    "mfa_replica_rebuild_counts": (i32, [vp, P(i64)]),
}
NKFAM = 9

_lib = None


def load_library(path=None):
    """Loads the CUDA library (raises if it is missing: no fallback exists)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(
            "mfa_brush_gb300: %s is missing; build it with `python -m mfa_brush_gb300.build` "
            "(nvcc, sm_103a). There is no CPU fallback." % p)
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


class MfaError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "MFA_ERR"), code, msg))
        self.code = code


def check(code, ctx=None):
    if code != MFA_OK:
        msg = ""
        if ctx is not None and ctx.value:
            msg = load_library().mfa_last_error(ctx).decode(errors="replace")
        raise MfaError(code, msg)
    return code


def dptr(a):
    """double* of a C-contiguous float64 numpy array (or None)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(dp)


def iptr(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ip)
