"""Host-side logic of the product (CPU only, no kernel launches): the C-ABI library loads and
exports every entry point include/mfa_gpu.h declares, the input parsers read the reference's own
deck, conf_old/conf_new round-trip, and the synthetic configurations are well formed."""
import os
import re

import numpy as np

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "mfa_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mfa_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.mfa_version().decode().startswith("mfa_gb300")


def test_abi_struct_sizes_match_header(lib):
    """ctypes mirrors of the structs must have the C sizes (checked through a round trip)."""
    import ctypes as C
    from mfa_brush_gb300 import abi
    o = abi.Options()
    lib.mfa_default_options(C.byref(o))
    assert (o.precision, o.skin, o.energy_every, o.use_graphs) == (abi.PREC_MIXED, 0.3, 10, 1)
    assert (o.profile_from_step, o.kspace_plain_sums) == (0, 0)


def test_struct_layouts_match_the_c_compiler(tmp_path):
    """Sizes of the ctypes mirrors against the C compiler's sizeof of the header's structs."""
    import ctypes as C
    import subprocess
    from mfa_brush_gb300 import abi
    names = {"mfa_inputs": abi.Inputs, "mfa_params": abi.Params, "mfa_system": abi.System,
             "mfa_options": abi.Options, "mfa_energies": abi.Energies, "mfa_observables": abi.Observables,
             "mfa_virial": abi.Virial, "mfa_averages": abi.Averages}
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "mfa_gpu.h"\nint main(void) {\n' +
                   "".join('  printf("%%zu\\n", sizeof(%s));\n' % n for n in names) + "  return 0;\n}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == [C.sizeof(t) for t in names.values()]


def test_header_flags(try_dir):
    from mfa_brush_gb300 import md
    f = md.flags_from_header(os.path.join(try_dir, "control_simulation.h"))
    assert (f.system, f.wall, f.solvent, f.thermostat, f.bin_type) == (0, 2, 3, 0, 0)
    assert (f.bending, f.orientation, f.brush_in_good_sv, f.poiseuille, f.particle_4) == (1, 1, 1, 0, 0)
    assert f.dpd_cut_off == 2.24 and f.force_switch_on == 1 and f.profiles == 1


def test_read_deck(try_deck):
    inp, p, s, a_type, r0, v, a = try_deck
    assert (inp.n_mon, inp.n_chain, inp.n_cell_w_x, inp.n_cell_w_y) == (10, 300, 30, 20)
    assert (inp.n_mon_d, inp.n_chain_d) == (1, 3000)
    assert inp.delta_sig[0] == 1.0 and (inp.a_w, inp.sigma_w) == (-3.2, 1.0)
    assert (inp.s_time, inp.n_relax, inp.n_obser, inp.n_safe) == (2, 0, 500000, 1000)
    assert inp.dt == 2e-4 and inp.temp == 0.8 and inp.z_space_wall == 40.0
    assert inp.mass_type[3] == 50.0 and inp.epsil[0] == 0.0 and abs(inp.epsil[2] - 0.333) < 1e-15
    assert (inp.k_bend, inp.alpha_eq, inp.iseed, inp.k_chain, inp.r_chain) == (80.0, 0.0, 311500357, 30.0, 1.5)
    assert list(inp.f_twall) == [2, 2, 1]
    assert np.bincount(a_type).tolist() == [0, 300, 2700, 3000]
    assert r0[0].tolist() == [24.249925, 1.0, 38.8]
    assert r0[:, 2].min() > 0 and r0[:, 2].max() < 40


def test_conf_round_trip(try_deck, tmp_path):
    from mfa_brush_gb300 import md
    inp, p, s, a_type, r0, v, a = try_deck
    path = str(tmp_path / "conf_new")
    md.write_conf_new(path, inp, a_type, r0, v, a)
    t2, r2, v2, a2 = md.read_conf_old(path, s.n_part)
    assert np.array_equal(t2, a_type)
    # f13.7 / f15.7 formats keep 7 decimals
    assert np.abs(r2 - r0).max() < 5.1e-8 and np.abs(v2 - v).max() < 5.1e-8 and np.abs(a2 - a).max() < 5.1e-8


def test_conf_new_writer_reproduces_the_reference_file(try_deck, tmp_path):
    """The restart file that the reference's try/ run wrote (store_config.f90:14-63, implicit
    walls), read and written back by the library: byte for byte the same file."""
    import gzip

    from conftest import GOLDEN
    from mfa_brush_gb300 import md
    inp, p, s, _, _, _, _ = try_deck
    with gzip.open(os.path.join(GOLDEN, "try", "conf_new.gz"), "rb") as g:
        ref = g.read()
    src = tmp_path / "conf_new_ref"
    src.write_bytes(ref)
    t, r, v, a = md.read_conf_old(str(src), s.n_part)
    out = tmp_path / "conf_new"
    md.write_conf_new(str(out), inp, t, r, v, a)
    assert out.read_bytes() == ref


def test_conf_new_explicit_walls_round_trip(tmp_path):
    """WALL 1: the wall beads' equilibrium positions (store_config.f90:47-52) follow the
    accelerations, one line per wall bead, before the eight lines of the top/bottom wall block;
    the file reads back with the same types and positions."""
    from mfa_brush_gb300 import configs, md
    inp = configs.wca_inputs(wall=1, dpd_cut_off=1.0)
    s, a_type, r0, v = configs.explicit_wall_channel(seed=2)
    inp.n_mon, inp.n_chain = s.n_mon, s.n_chain
    inp.n_mon_d, inp.n_chain_d = s.n_mon_d, s.n_chain_d
    n_wall = s.n_part - s.n_mon_tot
    assert n_wall > 0
    a = np.zeros_like(r0)
    path = tmp_path / "conf_new"
    md.write_conf_new(str(path), inp, a_type, r0, v, a)
    lines = path.read_text().splitlines()
    assert len(lines) == 4 + 3 * s.n_part + n_wall + 8
    walls = np.array([[float(x) for x in ln.split()] for ln in lines[4 + 3 * s.n_part:4 + 3 * s.n_part + n_wall]])
    assert np.abs(walls - r0[s.n_mon_tot:]).max() < 5.1e-8
    t2, r2, _, _ = md.read_conf_old(str(path), s.n_part)
    assert np.array_equal(t2, a_type) and np.abs(r2 - r0).max() < 5.1e-8


def test_unsupported_flags_are_rejected(try_deck):
    import ctypes as C
    from mfa_brush_gb300 import abi, md
    inp = try_deck[0]
    bad = abi.Inputs.from_buffer_copy(inp)
    bad.flags.symmetry = 1
    p, s = abi.Params(), abi.System()
    assert abi.load_library().mfa_derive_params(C.byref(bad), C.byref(p), C.byref(s)) == -9


def test_init_without_gpu_fails_loudly(try_deck):
    """On a machine without a GPU the context refuses to start (no CPU fallback)."""
    from mfa_brush_gb300 import abi, md
    if md.device_count() > 0:
        return
    inp, p, s, a_type, r0, v, a = try_deck
    try:
        md.MdSystem(p, s, a_type, r0, v, a)
    except abi.MfaError as e:
        assert e.code == -10
    else:
        raise AssertionError("context created without a device")


def test_replica_workload_shapes():
    from mfa_brush_gb300 import configs
    shapes = configs.draw_replica_shapes(256, 2024)
    sg, N, D, L = map(np.array, zip(*shapes))
    assert sg.min() >= 0.05 and sg.max() <= 0.3 and N.min() >= 10 and N.max() <= 100
    assert D.min() >= 10 and D.max() <= 40 and L.min() >= 15 and L.max() <= 40
    assert np.all(2 * sg * N <= 0.7 * 0.8 * D)


def test_generated_bonds_stay_clear_of_the_fene_limit():
    """The lattice spacing is capped at 1 sigma, so a chain's face-diagonal step is a bond of at
    most sqrt(2) sigma (the FENE limit is 1.5 sigma; at 1.49 the start's bond force is ~4000) and
    no two beads start closer than ~0.94 sigma: 16 replicas of the bench set and the melt."""
    from scipy.spatial import cKDTree
    from mfa_brush_gb300 import configs
    reps = configs.replicas(256, 2024, indices=list(range(0, 256, 16)))
    melt = configs.melt_brush(L=20.0, D=40.0)[1]
    for s, a_type, r0, v in reps + [melt]:
        L = np.array(list(s.boundary))
        for st, nc, nm in ((0, s.n_chain, s.n_mon), (s.n_chain * s.n_mon, s.n_chain_d, s.n_mon_d)):
            if nc == 0 or nm < 2:
                continue
            idx = st + np.arange(nc * nm).reshape(nc, nm)
            d = r0[idx[:, 1:]] - r0[idx[:, :-1]]
            d[..., :2] -= L[:2] * np.round(d[..., :2] / L[:2])
            assert np.sqrt((d ** 2).sum(-1)).max() <= np.sqrt(2.0) + 1e-9
        x = np.column_stack([r0[:, 0] % L[0], r0[:, 1] % L[1], r0[:, 2]])
        dd, _ = cKDTree(x, boxsize=[L[0], L[1], 1e9]).query(x, k=2)
        assert dd[:, 1].min() > 0.9


def test_small_channel_is_well_formed():
    from mfa_brush_gb300 import configs
    s, a_type, r0, v = configs.small_channel()
    L = s.boundary[0]
    assert s.n_part == len(a_type) == len(r0) and s.n_mon_tot == s.n_part
    assert abs(s.n_part - 0.8 * 20 ** 3) <= 1
    assert np.all((r0[:, 2] >= configs.Z_LO - 1e-12) & (r0[:, 2] <= s.boundary[2] - configs.Z_LO + 1e-12))
    assert np.all(a_type[: s.n_mon * s.n_chain : s.n_mon] == 1)
    nb = s.n_mon * s.n_chain
    d = r0[1:nb] - r0[: nb - 1]
    d[:, :2] -= L * np.round(d[:, :2] / L)
    keep = np.ones(nb - 1, bool)
    keep[s.n_mon - 1 :: s.n_mon] = False
    bl = np.linalg.norm(d[keep], axis=1)
    assert bl.max() < 1.5 and bl.min() > 0.9


def test_skin_tuner_sample_spans_the_set():
    from mfa_brush_gb300 import tune
    reps = list(range(256))
    s = tune.sample_replicas(reps, 32)
    assert len(s) == 32 and s[0] == 0 and s[-1] == 255 and s == sorted(s)
    assert tune.sample_replicas(reps[:5], 32) == reps[:5]


def _range_table(p):
    from mfa_brush_gb300 import abi
    return np.array([[p.range_2[i * abi.MAXT + j] for j in range(p.n_type)] for i in range(p.n_type)])


def test_charged_brush_configuration(lib):
    """configs.charged_brush: neutral; -4 per chain spread over the 39 non-head beads; 1280 +1
    counterions stored last as the fourth species; every pair WCA (heads among themselves off);
    slab Ewald switches."""
    from mfa_brush_gb300 import configs
    p, (s, a_type, r0, v) = configs.charged_brush()
    q = np.array([p.charge[t - 1] for t in a_type])
    assert s.n_part == 33600 and abs(q.sum()) < 1e-9
    assert np.count_nonzero(q) == 13760 and np.count_nonzero(q > 0) == 1280
    assert s.n_chain_e == 1280 and s.n_mon_e == 1 and np.all(a_type[-1280:] == 4)
    assert np.all(a_type[s.n_mon * s.n_chain: s.n_part - 1280] == 3)
    wca = (2.0 ** (1.0 / 6.0)) ** 2
    rt = _range_table(p)
    assert rt[0, 0] == 0.0 and np.allclose(rt.ravel()[1:], wca, rtol=1e-6)
    assert p.flags.system == 3 and p.flags.particle_4 == 1 and abs(p.alpha_c - 0.81) < 1e-15
    assert abs(p.rc_coul_2 - 9.0) < 1e-12 and p.n_kmax == 12


def test_melt_brush_tables_and_generation(lib):
    """configs.melt_brush: brush-melt and melt-melt cut at 2 * 2^(1/6) sigma with eps_bm = 1.2
    (x4 in the tables), brush-brush WCA, cosine bending on both chain kinds; a reduced box
    builds with every bond inside the FENE range."""
    from mfa_brush_gb300 import abi, configs
    p, (s, a_type, r0, v) = configs.melt_brush(L=20.0)
    c6 = 2.0 ** (1.0 / 6.0)
    rt = _range_table(p)
    assert np.isclose(rt[1, 1], c6 ** 2) and np.isclose(rt[0, 1], c6 ** 2)
    assert np.isclose(rt[1, 2], (2 * c6) ** 2) and np.isclose(rt[2, 2], (2 * c6) ** 2)
    assert np.isclose(p.epsil[1 * abi.MAXT + 2], 4.8) and np.isclose(p.epsil[2 * abi.MAXT + 2], 4.0)
    assert p.flags.bending == 1 and p.flags.bending_melt == 1 and p.bend_form == 1 and p.k_bend == 2.0
    assert s.n_mon_d == 20 and s.n_chain_d > 0 and abs(s.n_part - 0.85 * 20 * 20 * 40) <= 20
    L = s.boundary[0]
    for n0, n_mon, n_ch in ((0, s.n_mon, s.n_chain), (s.n_mon * s.n_chain, s.n_mon_d, s.n_chain_d)):
        c = r0[n0: n0 + n_mon * n_ch].reshape(n_ch, n_mon, 3)
        d = np.diff(c, axis=1)
        d[..., :2] -= L * np.round(d[..., :2] / L)
        assert np.linalg.norm(d, axis=2).max() < 1.5


def test_fp32_peak_probe_without_a_device(lib):
    """mfa_fp32_fma_peak reports MFA_ERR_NO_DEVICE where no GPU is visible, and rejects a null
    output pointer."""
    import ctypes as C
    from mfa_brush_gb300 import md
    out = C.c_double(0.0)
    assert lib.mfa_fp32_fma_peak(0, None) == -1  # MFA_ERR_ARG
    if md.device_count() < 1:
        assert lib.mfa_fp32_fma_peak(0, C.byref(out)) == -10  # MFA_ERR_NO_DEVICE

