"""Error budget of a tensor-core structure factor, emulated on the CPU.

The structure factor is the one k-space step that is a matrix product: with the phase tables
X(p, n) = exp(i n 2 pi x_p / L_x) (n >= 0), Y(p, m), Z(p, l), the k-set's (m, l) rows and
A(row, p) = q_p Y(p, m) Z(p, l),

  rho(row, +n) = sum_p A(row, p) X(p, n),   rho(row, -n) = sum_p A(row, p) conj X(p, n),

i.e. four real products P1 = Ar Xr, P2 = Ai Xi, P3 = Ar Xi, P4 = Ai Xr with M = rows, N = |n|
slots and K = the charged particles, which is how the CUDA kernel computes it on the FMA pipe
(FP32, plain sums over 32-particle tiles, compensated across them).  A tcgen05 form would take
its operands in a tensor-core format with FP32 accumulation: TF32 (10 mantissa bits) or BF16 (7),
alone or split into a sum of pieces (3xTF32: hi*hi + hi*lo + lo*hi; 3xBF16 the same with two BF16
pieces; 6xBF16 with three pieces and the six products of order <= 2).  This module rounds the
operands the way those formats do (round to nearest even on the mantissa), multiplies and
accumulates in FP32, and measures the k-space energy and forces that follow from each rho
against FP64 (the energy and forces are then formed in FP64, so the numbers are the structure
factor's share alone).  The mixed-precision force gate is 1e-5 of the force scale."""
import numpy as np
import pytest

FORMATS = ("fp32", "tf32", "bf16", "3xtf32", "3xbf16", "6xbf16")


def round_mantissa(x, bits):
    """float32 array rounded to `bits` explicit mantissa bits, round to nearest even."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    shift = 23 - bits
    bias = ((u >> np.uint64(shift)) & np.uint64(1)) + np.uint64((1 << (shift - 1)) - 1)
    u = (u + bias) & np.uint64(0xFFFFFFFF & ~((1 << shift) - 1))
    return u.astype(np.uint32).view(np.float32)


def split(x, bits, pieces):
    out, rest = [], np.asarray(x, np.float32)
    for _ in range(pieces):
        h = round_mantissa(rest, bits)
        out.append(h)
        rest = (rest - h).astype(np.float32)  # exact: h is rest rounded
    return out


def emulated_matmul(a, b, fmt, kchunk=None):
    """a (M, K) @ b (K, N) with the operands in `fmt` and FP32 accumulation; float64 result.  With
    kchunk, FP32 accumulation runs over chunks of kchunk along K and the chunks' sums are added in
    FP64 (the CUDA kernel's tiles of 32 particles; a tensor-core kernel's accumulator drained to
    FP64 every kchunk)."""
    if fmt == "fp64":
        return a @ b
    if kchunk:
        out = np.zeros((a.shape[0], b.shape[1]))
        for k0 in range(0, a.shape[1], kchunk):
            out += emulated_matmul(a[:, k0:k0 + kchunk], b[k0:k0 + kchunk], fmt)
        return out
    a32, b32 = a.astype(np.float32), b.astype(np.float32)
    if fmt == "fp32":
        return (a32 @ b32).astype(np.float64)
    bits = 10 if "tf32" in fmt else 7
    if fmt in ("tf32", "bf16"):
        return (round_mantissa(a32, bits) @ round_mantissa(b32, bits)).astype(np.float64)
    pieces, order = {"3xtf32": (2, 1), "3xbf16": (2, 1), "6xbf16": (3, 2)}[fmt]
    sa, sb = split(a32, bits, pieces), split(b32, bits, pieces)
    acc = np.zeros((a.shape[0], b.shape[1]), np.float32)
    terms = [(i, j) for i in range(pieces) for j in range(pieces) if i + j <= order]
    for i, j in sorted(terms, key=lambda t: -(t[0] + t[1])):  # the smallest terms first
        acc = (acc + sa[i] @ sb[j]).astype(np.float32)
    return acc.astype(np.float64)


def kspace_setup(r, L, kvec):
    """Integer (n, m, l) of every k-vector (slab geometry: z period 3 L_z) and the phase angles."""
    Lz = 3.0 * L[2]
    kint = np.rint(kvec * np.array([L[0], L[1], Lz]) / (2.0 * np.pi)).astype(int)
    assert np.allclose(kint * 2.0 * np.pi / np.array([L[0], L[1], Lz]), kvec, atol=1e-9)
    theta = 2.0 * np.pi * r / np.array([L[0], L[1], Lz])
    return kint, theta


def structure_factor(theta, q, kint, fmt, kchunk=None):
    """rho_k of every k of the k-set through the (rows x slots) product in `fmt`."""
    nxm = np.abs(kint[:, 0]).max()
    nym, nzm = np.abs(kint[:, 1]).max(), np.abs(kint[:, 2]).max()
    ctype = np.complex128 if fmt == "fp64" else np.complex64
    X = np.exp(1j * np.outer(theta[:, 0], np.arange(nxm + 1))).astype(ctype)
    Y = np.exp(1j * np.outer(theta[:, 1], np.arange(-nym, nym + 1))).astype(ctype)
    Z = np.exp(1j * np.outer(theta[:, 2], np.arange(-nzm, nzm + 1))).astype(ctype)
    rows, row_of = np.unique(kint[:, 1:], axis=0, return_inverse=True)
    row_of = row_of.ravel()
    A = (q.astype(ctype)[None, :] * Y[:, rows[:, 0] + nym].T * Z[:, rows[:, 1] + nzm].T).astype(ctype)
    Ar, Ai = A.real.astype(np.float64), A.imag.astype(np.float64)
    Xr, Xi = X.real.astype(np.float64), X.imag.astype(np.float64)
    P1, P2 = emulated_matmul(Ar, Xr, fmt, kchunk), emulated_matmul(Ai, Xi, fmt, kchunk)
    P3, P4 = emulated_matmul(Ar, Xi, fmt, kchunk), emulated_matmul(Ai, Xr, fmt, kchunk)
    n = kint[:, 0]
    an = np.abs(n)
    plus = (P1 - P2)[row_of, an] + 1j * (P3 + P4)[row_of, an]
    minus = (P1 + P2)[row_of, an] + 1j * (P4 - P3)[row_of, an]
    return np.where(n >= 0, plus, minus)


def energy_and_forces(r, q, kvec, rho, alpha, chunk=2048):
    """sum_k G(k) |rho_k|^2 and F_p = q_p sum_k G(k) k Im(conj(rho_k) e^{i k r_p}), FP64 (the
    oracle's k-space sum without its constant factors, which cancel in relative errors)."""
    k2 = (kvec ** 2).sum(1)
    G = np.exp(-k2 / (4.0 * alpha)) / k2
    U = float((G * np.abs(rho) ** 2).sum())
    F = np.zeros_like(r)
    for s in range(0, len(r), chunk):
        ph = r[s:s + chunk] @ kvec.T
        w = G * (np.cos(ph) * rho.imag - np.sin(ph) * rho.real)
        F[s:s + chunk] = q[s:s + chunk, None] * (w @ kvec)
    return U, F


def split_precision_errors(r, q, L, kvec, alpha, formats=FORMATS, kchunk=None):
    """{format: (relative energy error, max |dF| / F_rms)} of the structure factor in each format."""
    kint, theta = kspace_setup(r, L, kvec)
    U0, F0 = energy_and_forces(r, q, kvec, structure_factor(theta, q, kint, "fp64"), alpha)
    frms = np.sqrt(np.mean((F0 ** 2).sum(1)))
    out = {}
    for fmt in formats:
        U, F = energy_and_forces(r, q, kvec, structure_factor(theta, q, kint, fmt, kchunk), alpha)
        out[fmt] = (abs(U - U0) / abs(U0), np.linalg.norm(F - F0, axis=1).max() / frms)
    return out


def _charged_case(oracle_mod):
    from mfa_brush_gb300 import configs, md
    inp = configs.wca_inputs(gamma=1.0, thermostat=0)
    inp.flags.system = 3
    inp.charge[1], inp.charge[2] = -1.0, 1.0
    inp.alpha_c, inp.n_kmax, inp.rc_coul = 0.81, 8, 3.0
    p, _ = md.derive(inp)
    s, a_type, r0, v = configs.brush_channel(14.0, 12.0, 0.08, 10, rho=0.6, seed=21)
    o = oracle_mod.Oracle(p, s, a_type, r0, v)
    kvec = o.kvecs()
    o.close()
    charge = np.array([p.charge[t - 1] for t in range(1, 5)])
    q = charge[a_type[:s.n_mon_tot] - 1]
    m = q != 0
    return r0[:s.n_mon_tot][m], q[m], np.array(list(s.boundary)), kvec, p.alpha_c


def test_split_precision_error_budget(oracle_mod):
    """A brush channel with every bead charged (14 x 14 x 12, 1,400 charges, n_kmax 8), FP32
    accumulation over 32-particle chunks summed in FP64: FP32 operands meet the 1e-5 force gate by
    an order; a single TF32 or BF16 pass misses it; the 3xTF32 and 6xBF16 splits are back at the
    FP32 level."""
    r, q, L, kvec, alpha = _charged_case(oracle_mod)
    err = split_precision_errors(r, q, L, kvec, alpha, kchunk=32)
    for fmt, (eu, ef) in err.items():
        print("%-7s energy %.2e  force %.2e" % (fmt, eu, ef))
    assert err["fp32"][1] < 2e-6
    assert err["tf32"][1] > 1e-5 and err["bf16"][1] > err["tf32"][1]
    assert err["3xtf32"][1] < 1e-5 and err["6xbf16"][1] < 1e-5
    assert err["3xbf16"][1] > err["3xtf32"][1]


def test_round_mantissa_matches_the_formats():
    x = np.array([1.0 + 2.0 ** -11, 1.0 + 3 * 2.0 ** -11, 1.0 + 2.0 ** -8 + 2.0 ** -9, -3.0e-3],
                 np.float32)
    t = round_mantissa(x, 10)
    assert t[0] == 1.0 and t[1] == np.float32(1.0 + 2.0 ** -9)  # ties to even
    b = round_mantissa(x, 7)
    assert b[2] == np.float32(1.0 + 2.0 ** -7)  # tie rounds up to even
    h, lo = split(x, 10, 2)
    assert np.all(np.abs((h.astype(np.float64) + lo) - x) <= 2.0 ** -21 * np.abs(x))


@pytest.mark.parametrize("fmt", ["fp64", "fp32", "3xtf32"])
def test_emulated_matmul_shapes(fmt):
    rng = np.random.default_rng(1)
    a, b = rng.normal(size=(5, 40)), rng.normal(size=(40, 3))
    c = emulated_matmul(a, b, fmt)
    assert c.shape == (5, 3) and np.abs(c - a @ b).max() < 1e-4
