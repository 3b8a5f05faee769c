// mfa_forces.cu -- force kernels of the MD-DPD step.
//
// k_pair   : fluid_fluid.f90:97-261 with dpd_forces.f90:45-115 and ewald_real.f90:15-33 fused.
//            One thread per particle walks its full Verlet list (no atomics, no Newton-3 scatter);
//            each unordered pair is therefore evaluated from both sides, and the DPD noise is a
//            Philox draw keyed on (seed, step, min tag, max tag) so both sides see the same g and
//            momentum is conserved exactly in exact arithmetic.  Energies are halved per visit
//            (a fixed wall bead has no list: its pairs count in full).
//            MIXED: positions are fixed-point int4 (the int32 difference is the x,y minimum image),
//            all pair arithmetic is FP32.  In the fused mixed step the FP32 partial sums over each
//            batch of kept pairs go into an FP64 per-particle total, with the particle's bonded
//            terms (evaluated by the same thread), its 9-3 wall force and the body force; in the
//            drop-in the FP32 sum is added to the FP64 force.  With a single cut-off for every
//            type pair the screening compares against one constant (UNI).  With energies, the
//            pair, bond, angle and wall virial is summed as well.
// k_bonded : intra_molec.f90:16-188 (FENE), bending.f90:19-121 / bending_melt.f90:22-108 and
//            orientation.f90:24-88.  Owner computes: the thread of bead m evaluates every bond,
//            angle and orientation term that acts on m (terms centred on m-1, m, m+1) and adds
//            its own share, so no two threads write one particle.  The body (bonded_of) is
//            shared with the fused pair kernel.
// k_wall   : fluid_wall.f90:77-125 (implicit 9-3 walls), FP64.
// k_cforce : constant_force.f90:17-21 (Poiseuille body force m*g on every non-head bead).
#include <type_traits>

#include "mfa_integ.cuh"

namespace mfa {

template <bool MIXED>
using real_t = typename std::conditional<MIXED, float, double>::type;

// A constant in the kernel's precision: the FP32 copy for MIXED, the double otherwise.
template <bool MIXED>
__device__ __forceinline__ real_t<MIXED> cst(double d, float f) {
  if constexpr (MIXED) return f; else return d;
}

__device__ __forceinline__ double r2min_of(const SimConst& C, long long step) {
  if (!C.force_switch_on) return 0.;
  double r_time = (double)step * C.dt;
  return (r_time < C.r2min_time) ? (1. - r_time / C.r2min_time) * C.r2min_init : 0.;
}

// ---------------------------------------------------------------------------------------------
// Bonded terms
// ---------------------------------------------------------------------------------------------
template <bool MIXED>
struct BeadPos;
template <>
struct BeadPos<true> {
  int4 q;
  __device__ void load(const DevState& s, int slot) { q = __ldg(&s.pfx[slot]); }
};
template <>
struct BeadPos<false> {
  double x, y, z;
  __device__ void load(const DevState& s, int slot) { x = s.rx[slot]; y = s.ry[slot]; z = s.rz[slot]; }
};

// a - b with the x,y minimum image
template <bool MIXED>
__device__ __forceinline__ void bead_delta(const BeadPos<MIXED>& a, const BeadPos<MIXED>& b, const RepDesc& R,
                                           real_t<MIXED>* d) {
  if constexpr (MIXED) {
    d[0] = i2f_fast(fx_diff(a.q.x, b.q.x)) * R.ufx_f[0];
    d[1] = i2f_fast(fx_diff(a.q.y, b.q.y)) * R.ufx_f[1];
    d[2] = i2f_fast(fx_diff(a.q.z, b.q.z)) * R.ufx_f[2];
  } else {
    d[0] = mic_ref(a.x - b.x, R.L[0], R.invL[0]);
    d[1] = mic_ref(a.y - b.y, R.L[1], R.invL[1]);
    d[2] = a.z - b.z;
  }
}

// a * b rounded on its own, never merged into a multiply-add: a force term that the virial of an
// energy kernel also reads is rounded alike in the kernels with and without energies (whether the
// compiler merges a product into an add depends on the product's other uses)
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// One angle term of bending.f90:47-109 with r_prev = r_c - r_{c-1}, r_next = r_{c+1} - r_c.
// fa acts on c-1, fc on c+1 (c gets -fa-fc).  MIXED takes the angle's sine and cosine from
// |p x n| and p.n (the harmonic form its angle as atan2(|p x n|, p.n)), which keeps FP32
// accurate for the nearly straight chains that stiff brushes produce.
template <bool MIXED>
__device__ void bend_term(const real_t<MIXED>* rp, const real_t<MIXED>* rn, const SimConst& C, real_t<MIXED> kb,
                          real_t<MIXED> aeq, real_t<MIXED>* fa, real_t<MIXED>* fc, real_t<MIXED>& e) {
  using real = real_t<MIXED>;
  real dot = 0, rp2 = 0, rn2 = 0;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    dot += rn[j] * rp[j];
    rp2 += rp[j] * rp[j];
    rn2 += rn[j] * rn[j];
  }
  real dn[3], dp[3], dn2 = 0, dp2 = 0;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    dn[j] = rp[j] * rn2 - rn[j] * dot;
    dp[j] = -rn[j] * rp2 + rp[j] * dot;
    dn2 += dn[j] * dn[j];
    dp2 += dp[j] * dp[j];
  }
  const real small = cst<MIXED>(C.bend_small, C.bend_small_f);
  const real srp = sqrt(rp2), srn = sqrt(rn2);
  if (dn2 < small) {
    real u[3], nu = 0;
#pragma unroll
    for (int j = 0; j < 3; ++j) { u[j] = rp[j] / srp - rn[j] / srn; nu += u[j] * u[j]; }
    nu = sqrt(nu);
#pragma unroll
    for (int j = 0; j < 3; ++j) dn[j] = (nu != 0) ? u[j] / nu / srn : (real)0;
  } else {
    const real sc = (real)1 / sqrt(dn2 * rn2);
#pragma unroll
    for (int j = 0; j < 3; ++j) dn[j] *= sc;
  }
  if (dp2 < small) {
    real u[3], nu = 0;
#pragma unroll
    for (int j = 0; j < 3; ++j) { u[j] = rp[j] / srp - rn[j] / srn; nu += u[j] * u[j]; }
    nu = sqrt(nu);
#pragma unroll
    for (int j = 0; j < 3; ++j) dp[j] = (nu != 0) ? u[j] / nu / srp : (real)0;
  } else {
    const real sc = (real)1 / sqrt(dp2 * rp2);
#pragma unroll
    for (int j = 0; j < 3; ++j) dp[j] *= sc;
  }
  real fm;
  if constexpr (MIXED) {
    real cx = rp[1] * rn[2] - rp[2] * rn[1];
    real cy = rp[2] * rn[0] - rp[0] * rn[2];
    real cz = rp[0] * rn[1] - rp[1] * rn[0];
    const real cr = sqrtf(cx * cx + cy * cy + cz * cz);
    if (C.bend_form == 1) {
      // the cosine form needs sin(alpha) and cos(alpha) only: |p x n| / (|p| |n|) and
      // p.n / (|p| |n|), with no angle and no library sine (the force then takes the same
      // operations whether or not the energy is formed)
      const real inv = (real)1 / (srp * srn);
      fm = kb * (cr * inv);
      e = kb * ((real)1 - dot * inv);
    } else {
      const real da = atan2f(cr, dot) - aeq;
      fm = kb * da;
      e = (real)0.5 * fm * da;
    }
  } else {
    real ca = dot / sqrt(rp2 * rn2);
    const real alpha = (ca >= 1.0) ? aeq : acos(ca);  // bending.f90:93-98 guard: delta_alpha = 0
    if (C.bend_form == 1) {
      fm = kb * sin(alpha);
      e = kb * ((real)1 - cos(alpha));
    } else {
      real da = alpha - aeq;
      fm = kb * da;
      e = (real)0.5 * fm * da;
    }
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    fa[j] = mul_rn(fm, dp[j]);
    fc[j] = mul_rn(fm, dn[j]);
  }
}

// Virial partials of the bonded terms of one particle (EFLAG kernels): FENE, brush and melt
// bending as symmetric tensors (xx yy zz xy xz yz), orientation as a full one (row-major).
template <typename T>
struct BondVir {
  T fene[6], bend[6], bendm[6], orient[9];
  __device__ void zero() {
#pragma unroll
    for (int c = 0; c < 6; ++c) fene[c] = bend[c] = bendm[c] = 0;
#pragma unroll
    for (int c = 0; c < 9; ++c) orient[c] = 0;
  }
};

// Bonded force on the mobile particle i (owner computes, see k_bonded); adds to F[3] and, for the
// terms that i owns, to e4[4] = {FENE, brush bending, melt bending, orientation}.  With EFLAG the
// virial goes to bv: half of each of i's bonds (-fac d (x) d, the other half comes from the
// partner), the whole of the angle centred on i (-f_a (x) r_prev + f_c (x) r_next) and of the
// orientation term of a head (F_1 (x) (r_1 - r_head)).  Returns false when i is in no chain of two
// or more beads.
template <bool MIXED, bool EFLAG>
__device__ __forceinline__ bool bonded_of(const DevState& s, const SimConst& C, int mask, int i, int w,
                                          real_t<MIXED>* F, real_t<MIXED>* e4, BondVir<real_t<MIXED>>* bv) {
  using real = real_t<MIXED>;
  const RepDesc& R = s.reps[info_rep(w)];
  int kind = -1, m = 0, n = 0;
  const int t = __ldg(&s.tag[i]);
  const int lt = t - R.p0;
  if (lt < R.part_init_d) {
    kind = 0; n = R.n_mon; m = lt % n;
  } else if (lt < R.part_init_e) {
    kind = 1; n = R.n_mon_d; m = (lt - R.part_init_d) % n;
  } else if (lt < R.n_mon_tot) {
    kind = 2; n = R.n_mon_e; m = (lt - R.part_init_e) % n;
  }
  if (kind < 0 || n < 2) return false;
  const int t0 = t - m;
  {
    const bool do_fene = mask & 1;
    const bool do_bend = (kind == 0 && (mask & 2)) || (kind == 1 && (mask & 4));
    const bool do_or = kind == 0 && (mask & 8) && m <= 1;
    const int lo = max(0, m - ((do_bend) ? 2 : 1)), hi = min(n - 1, m + ((do_bend) ? 2 : 1));
    BeadPos<MIXED> P[5];  // beads m-2 .. m+2 (fixed slots, so the array stays in registers)
#pragma unroll
    for (int u = 0; u < 5; ++u) {
      const int b = m - 2 + u;
      if (b >= lo && b <= hi) P[u].load(s, __ldg(&s.slot_of_tag[t0 + b]));
    }
    if (do_fene) {
      const real kc = cst<MIXED>(C.k_chain, C.k_chain_f), ir2 = cst<MIXED>(C.inv_r_chain_2, C.inv_r_chain_2_f),
                 xm = cst<MIXED>(C.fene_xmax, C.fene_xmax_f);
      if (m > 0) {  // bond (m-1, m): this bead is the second partner
        real d[3];
        bead_delta<MIXED>(P[1], P[2], R, d);
        real x = (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) * ir2;
        x = x < xm ? x : xm;
        real fac = kc / ((real)1 - x) * ir2;
        F[0] += fac * d[0]; F[1] += fac * d[1]; F[2] += fac * d[2];
        if (EFLAG) sym_add(bv->fene, (real)-0.5 * fac, d[0], d[1], d[2]);
      }
      if (m < n - 1) {  // bond (m, m+1): first partner; energy counted here
        real d[3];
        bead_delta<MIXED>(P[2], P[3], R, d);
        real x = (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) * ir2;
        x = x < xm ? x : xm;
        real fac = kc / ((real)1 - x) * ir2;
        F[0] -= fac * d[0]; F[1] -= fac * d[1]; F[2] -= fac * d[2];
        if (EFLAG) {
          e4[0] += kc * ((real)-0.5 * log((real)1 - x));
          sym_add(bv->fene, (real)-0.5 * fac, d[0], d[1], d[2]);
        }
      }
    }
    if (do_bend) {
      const real kb = cst<MIXED>(C.k_bend, C.k_bend_f), aeq = cst<MIXED>(C.alpha_eq, C.alpha_eq_f);
#pragma unroll
      for (int u = 1; u <= 3; ++u) {  // the angle centred on bead c = m - 2 + u
        const int c = m - 2 + u;
        if (c < 1 || c > n - 2) continue;
        real rp[3], rn[3], fa[3], fc[3], e;
        bead_delta<MIXED>(P[u], P[u - 1], R, rp);
        bead_delta<MIXED>(P[u + 1], P[u], R, rn);
        bend_term<MIXED>(rp, rn, C, kb, aeq, fa, fc, e);
        if (u == 3) { F[0] += fa[0]; F[1] += fa[1]; F[2] += fa[2]; }
        else if (u == 2) {
          F[0] -= fa[0] + fc[0]; F[1] -= fa[1] + fc[1]; F[2] -= fa[2] + fc[2];
          if (EFLAG) {
            if (kind == 0) e4[1] += e; else e4[2] += e;
            real* wb = (kind == 0) ? bv->bend : bv->bendm;
            const int ia[6] = {0, 1, 2, 0, 0, 1}, ib[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
            for (int c = 0; c < 6; ++c) wb[c] += fc[ia[c]] * rn[ib[c]] - fa[ia[c]] * rp[ib[c]];
          }
        } else { F[0] += fc[0]; F[1] += fc[1]; F[2] += fc[2]; }
      }
    }
    if (do_or) {
      // orientation.f90:35-88: ghost bond head -> head -/+ z, against bond 1
      const BeadPos<MIXED> H = (m == 0) ? P[2] : P[1];   // the head
      const BeadPos<MIXED> B1 = (m == 0) ? P[3] : P[2];  // bead 1 of the chain
      real rp[3], rn[3];
      bead_delta<MIXED>(B1, H, R, rn);
      double hz;
      if constexpr (MIXED) hz = (double)H.q.z * R.ufx[2]; else hz = H.z;
      if constexpr (MIXED) {
        rp[0] = 0; rp[1] = 0; rp[2] = (hz > R.L[2] / 2) ? -1.f : 1.f;
      } else {
        double g = (hz > R.L[2] / 2) ? hz + 1.0 : hz - 1.0;
        rp[0] = 0; rp[1] = 0; rp[2] = hz - g;
      }
      real dot = 0, rp2 = 0, rn2 = 0, dn[3], dn2 = 0;
#pragma unroll
      for (int j = 0; j < 3; ++j) { dot += rn[j] * rp[j]; rp2 += rp[j] * rp[j]; rn2 += rn[j] * rn[j]; }
#pragma unroll
      for (int j = 0; j < 3; ++j) { dn[j] = rp[j] * rn2 - rn[j] * dot; dn2 += dn[j] * dn[j]; }
      const real srp = sqrt(rp2), srn = sqrt(rn2);
      if (dn2 < cst<MIXED>(C.bend_small, C.bend_small_f)) {
        real u[3], nu = 0;
#pragma unroll
        for (int j = 0; j < 3; ++j) { u[j] = rp[j] / srp - rn[j] / srn; nu += u[j] * u[j]; }
        nu = sqrt(nu);
#pragma unroll
        for (int j = 0; j < 3; ++j) dn[j] = (nu != 0) ? u[j] / nu / srn : (real)0;
      } else {
        const real sc = (real)1 / sqrt(dn2 * rn2);
#pragma unroll
        for (int j = 0; j < 3; ++j) dn[j] *= sc;
      }
      real alpha;
      if constexpr (MIXED) {
        real cx = rp[1] * rn[2] - rp[2] * rn[1];
        real cy = rp[2] * rn[0] - rp[0] * rn[2];
        real cz = rp[0] * rn[1] - rp[1] * rn[0];
        alpha = atan2f(sqrtf(cx * cx + cy * cy + cz * cz), dot);
      } else {
        real ca = dot / sqrt(rp2 * rn2);
        alpha = (ca >= 1.0) ? 0. : acos(ca);
      }
      const real da = alpha - cst<MIXED>(C.alpha_or, C.alpha_or_f);
      const real fm = cst<MIXED>(C.k_or, C.k_or_f) * da;
      const real sgn = (m == 0) ? (real)-1 : (real)1;
      const real sf = sgn * fm;
      F[0] += mul_rn(sf, dn[0]); F[1] += mul_rn(sf, dn[1]); F[2] += mul_rn(sf, dn[2]);
      if (EFLAG && m == 0) {
        e4[3] += (real)0.5 * fm * da;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) bv->orient[3 * a + b] += fm * dn[a] * rn[b];
      }
    }
  }
  return true;
}

// Slots and values of a symmetric tensor (6 components) for obs_push.
template <typename T>
__device__ __forceinline__ void sym_slots(int* sl, T* v, int base, const T* w6) {
  const int idx[6] = {0, 4, 8, 1, 2, 5};
#pragma unroll
  for (int c = 0; c < 6; ++c) { sl[c] = base + idx[c]; v[c] = w6[c]; }
}

// Slots and values of the bonded energies and virial tensors for obs_push (31 of them; terms
// that are off contribute zeros, which add nothing).
template <typename T>
__device__ __forceinline__ void bonded_slots(int* sl, T* v, const T* e4, const BondVir<T>& bv) {
  sl[0] = O_VINTRA; v[0] = e4[0];
  sym_slots(sl + 1, v + 1, O_VIR + 9 * V_FENE, bv.fene);
  sl[7] = O_VBEND; v[7] = e4[1];
  sym_slots(sl + 8, v + 8, O_VIR + 9 * V_BEND, bv.bend);
  sl[14] = O_VBENDM; v[14] = e4[2];
  sym_slots(sl + 15, v + 15, O_VIR + 9 * V_BENDM, bv.bendm);
  sl[21] = O_VOR; v[21] = e4[3];
#pragma unroll
  for (int c = 0; c < 9; ++c) { sl[22 + c] = O_VIR + 9 * V_OR + c; v[22 + c] = bv.orient[c]; }
}

template <bool MIXED, bool EFLAG>
__global__ void __launch_bounds__(128) k_bonded(DevState s, SimConst C, int mask, Acc acc, bool to_f4) {
  using real = real_t<MIXED>;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool inside = i < s.N;
  const int w = inside ? __ldg(&s.info[i]) : 0;
  const int rep = info_rep(w);
  real F[3] = {0, 0, 0};
  real e4[4] = {0, 0, 0, 0};
  BondVir<real> bv;
  if (EFLAG) bv.zero();
  const bool has = inside && info_mobile(w) && bonded_of<MIXED, EFLAG>(s, C, mask, i, w, F, e4, &bv);
  if (has) {
    if (MIXED && to_f4) {  // fused step: FP32 force array
      float4 f = s.f4[i];
      f.x += (float)F[0];
      f.y += (float)F[1];
      f.z += (float)F[2];
      s.f4[i] = f;
    } else {
      s.fx[i] += (double)F[0];
      s.fy[i] += (double)F[1];
      s.fz[i] += (double)F[2];
    }
  }
  if (EFLAG) {
    int sl[31];
    real v[31];
    bonded_slots(sl, v, e4, bv);
    obs_push<real, 31>(acc, sl, v, rep, has);
  }
}

// kept pairs per batch (a thread screens its list until it has this many, then they are evaluated),
// and list entries screened per group (their loads are all in flight at once).  Measured on 256
// brush replicas (4.66 M particles, skin 0.5): groups of 2 / 3 / 4 / 8 entries gave a pair kernel
// of 0.574 / 0.582 / 0.583 / 0.648 ms with the evaluation loop not unrolled; unrolling it by 2 or
// 4 cost 4 % or 20 %.  With the batch in shared memory, the kernel with the integration in its
// tail took 0.598 / 0.586 / 0.586 / 0.588 / 0.597 / 0.607 ms at batches of 8 / 10 / 12 / 16 /
// 24 / 32 (groups of 2; 12 with groups of 4: 0.585).
constexpr int PAIR_BATCH = 12;
constexpr int PAIR_G = 2;

// Force factor fs of the pair (i, j) along d = r_i - r_j (LJ with the switch-on clamp, DPD with the
// pair's Philox noise, real-space Coulomb), fluid_fluid.f90:97-261, dpd_forces.f90:45-115,
// ewald_real.f90:15-33; with EFLAG the pair's share `half` of its energies.
template <bool MIXED, bool EFLAG>
__device__ __forceinline__ real_t<MIXED> pair_fs(const DevState& s, const SimConst& C,
                                                 const PairEntry<real_t<MIXED>>& e, real_t<MIXED> dx,
                                                 real_t<MIXED> dy, real_t<MIXED> dz, int wj, int j,
                                                 real_t<MIXED> vix, real_t<MIXED> viy, real_t<MIXED> viz, int tag_i,
                                                 int p0, uint32_t nkey, real_t<MIXED> r2min,
                                                 real_t<MIXED> half, real_t<MIXED>& e_lj, real_t<MIXED>& e_c) {
  using real = real_t<MIXED>;
  (void)wj;
  const real sig = cst<MIXED>(C.sig, C.sig_f), gam = cst<MIXED>(C.gamma, C.gamma_f);
  const real coul_rc2 = cst<MIXED>(C.coul_rc2, C.coul_rc2_f);
  const real r2raw = dx * dx + dy * dy + dz * dz;
  const int fl = e.flags;
  real r2 = r2raw;
  const bool in_lj = r2raw < e.range2;
  real fs = 0;  // force factor along d = r_i - r_j
  if (in_lj) {
    r2 = r2raw < r2min ? r2min : r2raw;
    // MIXED: the hardware reciprocal (2 ulp) instead of the IEEE division sequence
    real inv_r2;
    if constexpr (MIXED) inv_r2 = __fdividef(1.f, r2); else inv_r2 = (real)1 / r2;
    const real s2 = e.sig2 * inv_r2;
    const real s6 = s2 * s2 * s2;
    const real s12 = s6 * s6;
    fs = e.eps4 * ((real)12 * s12 - (real)6 * s6) * inv_r2;
    if (EFLAG) e_lj += half * e.eps4 * ((s12 - s6) - e.shift);
  }
  const bool dpd = (in_lj && (fl & PF_DPD_LJ)) || ((fl & PF_DPD_OWN) && r2 < e.dpd_rc2);
  if (dpd) {
    real vjx, vjy, vjz;
    int tag_j;
    if constexpr (MIXED) {
      float4 v4 = __ldg(&s.vf[j]);
      vjx = v4.x; vjy = v4.y; vjz = v4.z;
      tag_j = __float_as_int(v4.w) - p0;
    } else {
      dbl4 v4 = s.vd[j];
      vjx = v4.x; vjy = v4.y; vjz = v4.z;
      tag_j = (int)__double_as_longlong(v4.w) - p0;
    }
    real r, ir;
    if constexpr (MIXED) {  // one hardware reciprocal square root (2 ulp)
      ir = rsqrtf(r2);
      r = r2 * ir;
    } else {
      r = sqrt(r2);
      ir = (real)1 / r;
    }
    real wr, wd;
    if (C.dpd_weight1) {
      wr = wd = 1;
    } else {
      wr = (real)1 - r * ((fl & PF_DPD_OWN) ? e.inv_dpd_rc : e.inv_rc);
      wd = wr * wr;
    }
    real g;
    if constexpr (MIXED) g = pair_gauss_f(nkey, tag_i, tag_j);
    else g = pair_gauss_d(nkey, tag_i, tag_j);
    const real rdot = ((vix - vjx) * dx + (viy - vjy) * dy + (viz - vjz) * dz) * ir;
    fs += (sig * wr * g - gam * wd * rdot) * ir;
  }
  if (fl & PF_COUL) {
    const bool in_c = (coul_rc2 > 0) ? (r2raw < coul_rc2) : in_lj;
    if (in_c) {
      const real rc2 = in_lj ? r2 : r2raw;
      const real r = sqrt(rc2), ir = (real)1 / r;
      const real qq = e.qq;
      const real sqa = cst<MIXED>(C.sqrt_alpha, C.sqrt_alpha_f);
      const real ec = erfc(sqa * r);
      if (EFLAG) e_c += half * qq * ec * ir;
      const real isp = cst<MIXED>(C.inv_sqrt_pi, C.inv_sqrt_pi_f), ac = cst<MIXED>(C.alpha_c, C.alpha_c_f);
      fs += (qq * sqa * isp * (real)2 * exp(-ac * rc2) * ir + qq * ec * ir * ir) * ir;
    }
  }
  return fs;
}

// The pair kernel.  Template switches:
//   MIXED   FP32 pair arithmetic on the fixed-point views (else FP64 throughout);
//   EFLAG   energies and the virial into the accumulators;
//   FUSED   the fused mixed-precision step (MIXED only): FP32 partial sums over each batch of kept
//           pairs are added to an FP64 per-particle total, together with the bonded, wall and body
//           forces of the particle, and the total is stored (rounded to FP32) in the force array
//           that the integrator reads;
//   BONDED  (FUSED only) the particle's bonded terms (bonded_of) in the same thread, which saves
//           the bonded kernel's launch and its read-modify-write of the force;
//   UNI     (MIXED only) one screening cut-off for every type pair (SimConst::scr2_uni_f).
// Without FUSED the forces are added to (accumulate) or stored in the FP64 force arrays.
// Virial (EFLAG): each visit of a pair adds half of F_ij (x) (r_i - r_j) (the other visit adds the
// other half); a pair with a fixed wall bead, which has no list of its own, counts in full.
//   INTEG   (FUSED) the step's integration in the tail (with EFLAG also its kinetic energy and
//           tensor and the head forces, into the same warp reduction): each thread takes its
//           particle's force and runs the integrator's update (int_mixed_particle, MODE 2) on it,
//           writing the next step's views to the other view buffers (pfx_alt, vf_alt) while the
//           neighbours still read pfx and vf; wall beads copy their views across, and the step
//           counter of the other set is this one's plus one.  No force array is written.
//   PERSIST (FUSED only) a grid of the blocks that fit on the GPU at once; each block takes tiles
//           of blockDim.x particles from a queue (s.pair_q[0], one atomic ticket per tile, no
//           waiting) and the last block to finish resets the queue for the next launch.  Compiled
//           for 8 resident blocks per SM (64 registers): at 9 the tile loop spills.
template <bool MIXED, bool EFLAG, bool FUSED = false, bool BONDED = false, bool UNI = false, bool PERSIST = false,
          bool INTEG = false>
// Resident blocks per SM: 10 for the kernel with the integration in its tail (48 registers and a
// 52-byte spill; 0.558 against 0.584 ms per step at 9 blocks, 56 registers; 11 or 12 blocks leave
// 40 registers and spill 124 bytes: 0.579 ms), 9 for the other fused forms, 8 for the persistent
// schedule (its tile loop spills at 9).
__global__ void __launch_bounds__(128, MIXED ? (PERSIST ? 8 : ((INTEG && !EFLAG) ? 10 : 9)) : 4) k_pair(DevState s, SimConst C, bool accumulate,
                                                                             Acc acc, int bmask = 0) {
  using real = real_t<MIXED>;
  static_assert(!FUSED || MIXED, "the fused form is the mixed-precision one");
  static_assert(!BONDED || FUSED, "bonded terms are fused only into the fused form");
  static_assert(!INTEG || (FUSED && !PERSIST), "the integration is fused into the fused form");
  __shared__ PairEntry<real> tab[NPAIR];
  // FUSED: the particle's FP64 total, in shared memory while the pair loop runs (registers are
  // scarce there; it is touched once per batch)
  __shared__ double ftot[FUSED ? 3 : 1][FUSED ? 128 : 1];
  for (int k = threadIdx.x; k < NPAIR; k += blockDim.x) {
    if constexpr (MIXED) tab[k] = s.tabf[k]; else tab[k] = s.tabd[k];
  }
  __shared__ int tile_sh;
  const int ntile = (s.N + blockDim.x - 1) / blockDim.x;
  for (int pass = 0;; ++pass) {
  int tile;
  if constexpr (PERSIST) {
    __syncthreads();  // every thread is done with the previous tile's ticket
    if (threadIdx.x == 0) tile_sh = atomicAdd(s.pair_q, 1);
    __syncthreads();
    tile = tile_sh;
    if (tile >= ntile) break;
  } else {
    if (pass) break;
    tile = blockIdx.x;
  }
  const int i = tile * blockDim.x + threadIdx.x;
  const bool inside = i < s.N;
  const int w = inside ? __ldg(&s.info[i]) : 0;
  const bool active = inside && info_mobile(w);
  const int rep = info_rep(w);
  float e_w = 0.f, w_wall = 0.f;  // FUSED: wall energy and virial
  if constexpr (FUSED) {
    // the particle's external forces first: its FP64 total starts from them
    double ez = 0., ex = 0., ey = 0.;
    if (active) {
      const int ti = info_type(w);
      if (C.wall == 2) {  // fluid_wall.f90:96-121 from the FP64 position: distances to both walls
        const double zd = s.rz[i];
        const float zl = d2f_fast(zd), zh = d2f_fast(s.reps[rep].L[2] - zd);
        float fwb, fwt;
        wall93f_split(C, ti, zl, zh, fwb, fwt, e_w);
        ez = f2d_fast(fwb) + f2d_fast(fwt);
        if (EFLAG) w_wall = fwb * zl - fwt * zh;  // each wall's force times z - z_wall
      }
      if (C.poiseuille && ti != 0) {  // constant_force.f90:17-21: m g on every non-head bead
        ex = f2d_fast(C.mass_f[ti] * C.cforce_f[0]);
        ey = f2d_fast(C.mass_f[ti] * C.cforce_f[1]);
        ez += f2d_fast(C.mass_f[ti] * C.cforce_f[2]);
      }
    }
    ftot[0][threadIdx.x] = ex;
    ftot[1][threadIdx.x] = ey;
    ftot[2][threadIdx.x] = ez;
  }
  __syncthreads();
  // Shared memory of the batch of kept list entries (a column per thread) and, in the energy
  // variant with bonded terms, of the bonded virial partials after it: the batch is dead once
  // the pair loop ends, and a barrier separates the two uses, so the variant keeps room for L1.
  constexpr int JL_WORDS = PAIR_BATCH * 128;
  constexpr int BV_WORDS = (EFLAG && BONDED) ? 128 * (int)(sizeof(BondVir<real_t<MIXED>>) / 4) : 0;
  __shared__ __align__(16) int pair_pool[JL_WORDS > BV_WORDS ? JL_WORDS : BV_WORDS];
  real fx = 0, fy = 0, fz = 0;        // the current batch (FUSED), else the whole sum
  real e_lj = 0, e_c = 0;
  real wv[6] = {0, 0, 0, 0, 0, 0};   // EFLAG: pair virial, xx yy zz xy xz yz
  if (active) {
    const RepDesc& R = s.reps[rep];
    const long long step = R.s_time + *s.steps_done;
    const real r2min = C.force_switch_on ? (real)r2min_of(C, step) : (real)0;
    const int ti = info_type(w);
    const int n = __ldg(&s.nn[i]);
    const int p0 = R.p0;
    // own position / velocity
    int4 qi;
    dbl4 pi;
    real vix, viy, viz;
    int tag_i;
    real ux = 0, uy = 0, uz = 0;
    if constexpr (MIXED) {
      qi = __ldg(&s.pfx[i]);
      float4 v4 = __ldg(&s.vf[i]);
      vix = v4.x; viy = v4.y; viz = v4.z;
      tag_i = __float_as_int(v4.w) - p0;
      ux = R.ufx_f[0]; uy = R.ufx_f[1]; uz = R.ufx_f[2];
    } else {
      pi = s.pd[i];
      dbl4 v4 = s.vd[i];
      vix = v4.x; viy = v4.y; viz = v4.z;
      tag_i = (int)__double_as_longlong(v4.w) - p0;
    }
    const double L0 = R.L[0], L1 = R.L[1], iL0 = R.invL[0], iL1 = R.invL[1];
    const uint32_t nkey = pair_key(R.seed, step);  // the replica's noise key of this step
    const int* __restrict__ nb = s.nbr + i;
    auto delta = [&](int j, real& dx, real& dy, real& dz) -> int {
      if constexpr (MIXED) {
        const int4 qj = __ldg(&s.pfx[j]);
        dx = i2f_fast(fx_diff(qi.x, qj.x)) * ux;
        dy = i2f_fast(fx_diff(qi.y, qj.y)) * uy;
        dz = i2f_fast(fx_diff(qi.z, qj.z)) * uz;
        return qj.w;
      } else {
        const dbl4 pj = s.pd[j];
        dx = mic_ref(pi.x - pj.x, L0, iL0);
        dy = mic_ref(pi.y - pj.y, L1, iL1);
        dz = pi.z - pj.z;
        return (int)__double_as_longlong(pj.w);
      }
    };
    // Two phases per batch: (1) screen list entries with the cheap distance test and keep the
    // ones inside any interaction range, (2) evaluate LJ + DPD + Coulomb on the kept pairs only.
    // Without the split a warp runs the Philox/DPD body whenever any lane has an interacting
    // pair, i.e. on almost every list entry.
    constexpr int BATCH = PAIR_BATCH;
    constexpr int G = PAIR_G;  // list entries screened per group: their loads are all in flight at once
    // the batch's kept entries in shared memory, a column per thread (conflict-free): a
    // dynamically indexed local array lives in local memory, whose loads missed L1 behind the
    // gathers
    int* const jl = pair_pool + threadIdx.x;
    int k = 0;
    // screening against the largest cut-off of the type pair; MIXED uses the coarse conversion
    // (512 fixed-point units of resolution, inside the 2e-4 margin of screen2)
    const float cx = ux * 512.f, cy = uy * 512.f, cz = uz * 512.f;
    auto screen = [&](int j) -> bool {
      if constexpr (MIXED) {
        const int4 qj = __ldg(&s.pfx[j]);
        const float dx = i2f_coarse(fx_diff(qi.x, qj.x), 9) * cx;
        const float dy = i2f_coarse(fx_diff(qi.y, qj.y), 9) * cy;
        const float dz = i2f_coarse(fx_diff(qi.z, qj.z), 9) * cz;
        return dx * dx + dy * dy + dz * dz < (UNI ? C.scr2_uni_f : tab[ti * MAXT + info_type(qj.w)].screen2);
      } else {
        real dx, dy, dz;
        const int wj = delta(j, dx, dy, dz);
        return dx * dx + dy * dy + dz * dz < tab[ti * MAXT + info_type(wj)].screen2;
      }
    };
    while (k < n) {
      int m = 0;
      // groups of G independent entries (index loads first, then the position gathers)
      // (the next group's list indices are loaded one group ahead, hiding their DRAM latency)
      int jg[G];
      if (k + G <= n) {
#pragma unroll
        for (int u = 0; u < G; ++u) jg[u] = __ldg(nb + (size_t)(k + u) * s.Np);
      }
      while (k + G <= n && m <= BATCH - G) {
        int jn[G];
        const bool more = k + 2 * G <= n;
#pragma unroll
        for (int u = 0; u < G; ++u) jn[u] = more ? __ldg(nb + (size_t)(k + G + u) * s.Np) : 0;
        bool hg[G];
#pragma unroll
        for (int u = 0; u < G; ++u) hg[u] = screen(jg[u]);
#pragma unroll
        for (int u = 0; u < G; ++u)
          if (hg[u]) jl[128 * m++] = jg[u];
        k += G;
#pragma unroll
        for (int u = 0; u < G; ++u) jg[u] = jn[u];
      }
      while (k < n && m < BATCH) {
        const int j = __ldg(nb + (size_t)k * s.Np);
        ++k;
        if (screen(j)) jl[128 * m++] = j;
      }
#pragma unroll 1
      for (int t = 0; t < m; ++t) {
        const int j = jl[128 * t];
        real dx, dy, dz;
        const int wj = delta(j, dx, dy, dz);
        const PairEntry<real>& e = tab[ti * MAXT + info_type(wj)];
        // half of each mobile pair (both ends sum it); a fixed wall bead has no list of its own
        const real half = info_mobile(wj) ? (real)0.5 : (real)1;
        const real fs = pair_fs<MIXED, EFLAG>(s, C, e, dx, dy, dz, wj, j, vix, viy, viz, tag_i, p0, nkey,
                                              r2min, half, e_lj, e_c);
        if constexpr (MIXED) {  // unmerged products and sums: alike with and without energies
          fx = __fadd_rn(fx, __fmul_rn(fs, dx));
          fy = __fadd_rn(fy, __fmul_rn(fs, dy));
          fz = __fadd_rn(fz, __fmul_rn(fs, dz));
        } else {
          fx += fs * dx;
          fy += fs * dy;
          fz += fs * dz;
        }
        if (EFLAG) sym_add(wv, half * fs, dx, dy, dz);
      }
      if constexpr (FUSED) {  // the batch's FP32 partial into the FP64 total
        ftot[0][threadIdx.x] += f2d_fast(fx);
        ftot[1][threadIdx.x] += f2d_fast(fy);
        ftot[2][threadIdx.x] += f2d_fast(fz);
        fx = fy = fz = 0;
      }
    }
  }
  real eb[4] = {0, 0, 0, 0};
  // the bonded virial partials of the thread (EFLAG): in shared memory, where the bonded terms'
  // registers are scarce (27 words per thread: a stride prime to the 32 banks)
  __shared__ BondVir<real> bv_unused[1];  // the reference the other variants pass and never use
  BondVir<real>& bv = (EFLAG && BONDED) ? reinterpret_cast<BondVir<real>*>(pair_pool)[threadIdx.x] : bv_unused[0];
  if (EFLAG && BONDED) {
    __syncthreads();  // every thread of the block is past its pair loop: the batch area is free
    bv.zero();
  }
  bool hb = false;
  double fxd = 0., fyd = 0., fzd = 0.;
  // INTEG with EFLAG: the integrator's kinetic energy, kinetic tensor and head forces
  float ike = 0.f, ikin[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, ifh[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if constexpr (FUSED) {
    fxd = ftot[0][threadIdx.x];
    fyd = ftot[1][threadIdx.x];
    fzd = ftot[2][threadIdx.x];
    if (active) {
      if constexpr (BONDED) {
        real fb[3] = {0, 0, 0};
        hb = bonded_of<MIXED, EFLAG>(s, C, bmask, i, w, fb, eb, &bv);
        fxd += f2d_fast(fb[0]);
        fyd += f2d_fast(fb[1]);
        fzd += f2d_fast(fb[2]);
      }
    }
  }
  if (inside) {
    if constexpr (INTEG) {
      if (active) {
        int_mixed_particle<2, EFLAG>(s, C, i, w, d2f_fast(fxd), d2f_fast(fyd), d2f_fast(fzd), s.pfx_alt, s.vf_alt,
                                     ike, ikin, ifh);
      } else if (C.move_walls) {  // a wall bead on a moving wall: its next site
        double x, y, z;
        s.pfx_alt[i] = move_wall_bead(s, C, i, w, x, y, z);
        s.vf_alt[i] = s.vf[i];
      } else {  // a wall bead: its views as they are
        s.pfx_alt[i] = s.pfx[i];
        s.vf_alt[i] = s.vf[i];
      }
      if (i == 0) *s.steps_alt = *s.steps_done + 1;
    } else if constexpr (FUSED) {
      s.f4[i] = make_float4(d2f_fast(fxd), d2f_fast(fyd), d2f_fast(fzd), 0.f);
    } else if (accumulate) {
      if (active) {
        s.fx[i] += (double)fx;
        s.fy[i] += (double)fy;
        s.fz[i] += (double)fz;
      }
    } else {
      s.fx[i] = fx;
      s.fy[i] = fy;
      s.fz[i] = fz;
    }
  }
  if (EFLAG) {  // one warp reduction for every energy and virial component of the kernel
    constexpr int NB = BONDED ? 31 : 0, NW = FUSED ? 2 : 0, NI = INTEG ? 13 : 0, NV = 8 + NB + NW + NI;
    int sl[NV];
    real v[NV];
    sl[0] = O_VFF; v[0] = e_lj;
    sl[1] = O_VCOUL; v[1] = e_c;
    sym_slots(sl + 2, v + 2, O_VIR + 9 * V_PAIR, wv);
    if constexpr (BONDED) {
      (void)hb;
      bonded_slots(sl + 8, v + 8, eb, bv);
    }
    if constexpr (FUSED) {
      sl[8 + NB] = O_VFW; v[8 + NB] = e_w;
      sl[9 + NB] = O_VIR + 9 * V_WALL + 8; v[9 + NB] = w_wall;
    }
    if constexpr (INTEG) {  // the integrator's kinetic energy, kinetic tensor and head forces
      constexpr int b = 8 + NB + NW;
      const int idx[6] = {0, 4, 8, 1, 2, 5};
      sl[b] = O_TFLUID; v[b] = ike;
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        sl[b + 1 + c] = O_KIN + idx[c]; v[b + 1 + c] = ikin[c];
        sl[b + 7 + c] = O_FH + c; v[b + 7 + c] = ifh[c];
      }
    }
    obs_push<real, NV>(acc, sl, v, rep, active);
  }
  }
  if constexpr (PERSIST) {  // the last block out resets the queue (every block has drawn its last ticket)
    if (threadIdx.x == 0 && atomicAdd(s.pair_q + 1, 1) == (int)gridDim.x - 1) {
      s.pair_q[0] = 0;
      s.pair_q[1] = 0;
    }
  }
}

void launch_pair(const DevState& s, const SimConst& C, cudaStream_t st, bool accumulate, bool eflag, Acc acc,
                 int block, int bonded_mask, bool integ) {
  // 32, 64 or 128 threads per block (the kernel is compiled for at most 128); anything else
  // takes the built-in 128
  const int B = (block == 32 || block == 64) ? block : 128;
  const int g = (s.N + B - 1) / B;
  const bool uni = C.scr2_uni_f > 0.f;
  if (s.mixed && !accumulate) {  // the fused step
    using KernT = void (*)(DevState, SimConst, bool, Acc, int);
    // [bonded][uni][eflag]
    const KernT ks[2][2][2] = {{{k_pair<true, false, true>, k_pair<true, true, true>},
                                {k_pair<true, false, true, false, true>, k_pair<true, true, true, false, true>}},
                               {{k_pair<true, false, true, true>, k_pair<true, true, true, true>},
                                {k_pair<true, false, true, true, true>, k_pair<true, true, true, true, true>}}};
    // the persistent schedule for the steps without energies: [bonded][uni]
    const KernT kp[2][2] = {{k_pair<true, false, true, false, false, true>, k_pair<true, false, true, false, true, true>},
                            {k_pair<true, false, true, true, false, true>, k_pair<true, false, true, true, true, true>}};
    // with the step's integration in the tail: [eflag][bonded][uni]
    const KernT ki[2][2][2] = {{{k_pair<true, false, true, false, false, false, true>,
                                 k_pair<true, false, true, false, true, false, true>},
                                {k_pair<true, false, true, true, false, false, true>,
                                 k_pair<true, false, true, true, true, false, true>}},
                               {{k_pair<true, true, true, false, false, false, true>,
                                 k_pair<true, true, true, false, true, false, true>},
                                {k_pair<true, true, true, true, false, false, true>,
                                 k_pair<true, true, true, true, true, false, true>}}};
    const int bi = bonded_mask ? 1 : 0, ui = uni ? 1 : 0;
    if (integ) {
      ki[eflag ? 1 : 0][bi][ui]<<<g, B, 0, st>>>(s, C, false, acc, bonded_mask);
    } else if (s.pair_persist && !eflag) {
      const KernT k = kp[bi][ui];
      int per_sm = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, B, 0);
      const int grid = std::min(g, std::max(per_sm, 1) * s.nsm);
      k<<<grid, B, 0, st>>>(s, C, false, acc, bonded_mask);
    } else {
      ks[bi][ui][eflag ? 1 : 0]<<<g, B, 0, st>>>(s, C, false, acc, bonded_mask);
    }
  } else if (s.mixed) {  // the drop-in: added to the FP64 force
    if (eflag) k_pair<true, true><<<g, B, 0, st>>>(s, C, true, acc);
    else k_pair<true, false><<<g, B, 0, st>>>(s, C, true, acc);
  } else {
    if (eflag) k_pair<false, true><<<g, B, 0, st>>>(s, C, accumulate, acc);
    else k_pair<false, false><<<g, B, 0, st>>>(s, C, accumulate, acc);
  }
}

void launch_bonded(const DevState& s, const SimConst& C, cudaStream_t st, int mask, bool eflag, Acc acc,
                   bool fused) {
  if (!mask) return;
  int B = 128, g = (s.N + B - 1) / B;
  if (s.mixed) {
    if (eflag) k_bonded<true, true><<<g, B, 0, st>>>(s, C, mask, acc, fused);
    else k_bonded<true, false><<<g, B, 0, st>>>(s, C, mask, acc, fused);
  } else {
    if (eflag) k_bonded<false, true><<<g, B, 0, st>>>(s, C, mask, acc, false);
    else k_bonded<false, false><<<g, B, 0, st>>>(s, C, mask, acc, false);
  }
}

// ---------------------------------------------------------------------------------------------
// Implicit 9-3 walls and the constant body force
// ---------------------------------------------------------------------------------------------
template <bool EFLAG>
__global__ void k_wall(DevState s, SimConst C, Acc acc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool inside = i < s.N;
  const int w = inside ? s.info[i] : 0;
  const bool active = inside && info_mobile(w);
  double e = 0., wzz = 0.;
  if (active) {
    const RepDesc& R = s.reps[info_rep(w)];
    const double z = s.rz[i];
    double fb, ft;
    wall93_split(C, info_type(w), z, R.L[2], fb, ft, e);
    s.fz[i] += fb + ft;
    wzz = fb * z + ft * (z - R.L[2]);  // each wall's force times z - z_wall
  }
  if (EFLAG) {
    const int sl[2] = {O_VFW, O_VIR + 9 * V_WALL + 8};
    const double v[2] = {e, wzz};
    obs_push<double, 2>(acc, sl, v, info_rep(w), active);
  }
}

void launch_wall(const DevState& s, const SimConst& C, cudaStream_t st, bool eflag, Acc acc) {
  int B = 256, g = (s.N + B - 1) / B;
  if (eflag) k_wall<true><<<g, B, 0, st>>>(s, C, acc);
  else k_wall<false><<<g, B, 0, st>>>(s, C, acc);
}

__global__ void k_cforce(DevState s, SimConst C) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.N) return;
  const int w = s.info[i];
  if (!info_mobile(w) || info_type(w) == 0) return;
  const double m = C.mass[info_type(w)];
  s.fx[i] += m * C.const_force[0];
  s.fy[i] += m * C.const_force[1];
  s.fz[i] += m * C.const_force[2];
}

void launch_const_force(const DevState& s, const SimConst& C, cudaStream_t st) {
  int B = 256, g = (s.N + B - 1) / B;
  k_cforce<<<g, B, 0, st>>>(s, C);
}

// ---------------------------------------------------------------------------------------------
// Pair list export: every interacting pair (local tags, i<j) of replica `rep`, FP64 distances.
// ---------------------------------------------------------------------------------------------
__global__ void k_pair_list(DevState s, SimConst C, int rep, int* __restrict__ out, long long cap,
                            unsigned long long* __restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.N) return;
  const int w = s.info[i];
  if (info_rep(w) != rep || !info_mobile(w)) return;
  const RepDesc& R = s.reps[rep];
  const int ti = info_type(w), tgi = s.tag[i];
  const int n = s.nn[i];
  for (int k = 0; k < n; ++k) {
    int j = s.nbr[(size_t)k * s.Np + i];
    int wj = s.info[j];
    int tgj = s.tag[j];
    if (!info_mobile(wj) || tgj <= tgi) continue;
    double dx = mic_ref(s.rx[i] - s.rx[j], R.L[0], R.invL[0]);
    double dy = mic_ref(s.ry[i] - s.ry[j], R.L[1], R.invL[1]);
    double dz = s.rz[i] - s.rz[j];
    double r2 = dx * dx + dy * dy + dz * dz;
    const PairEntry<double>& e = s.tabd[ti * MAXT + info_type(wj)];
    bool hit = r2 < e.range2;
    if (!hit && (e.flags & PF_DPD_OWN)) hit = r2 < e.dpd_rc2;
    if (!hit && (e.flags & PF_COUL) && C.coul_rc2 > 0.) hit = r2 < C.coul_rc2;
    if (hit) {
      unsigned long long k2 = atomicAdd(count, 1ull);
      if ((long long)k2 < cap) {
        out[2 * k2] = tgi - R.p0;
        out[2 * k2 + 1] = tgj - R.p0;
      }
    }
  }
}

void launch_pair_list(const DevState& s, const SimConst& C, cudaStream_t st, int rep, int* pairs, long long cap,
                      unsigned long long* count) {
  int B = 128, g = (s.N + B - 1) / B;
  k_pair_list<<<g, B, 0, st>>>(s, C, rep, pairs, cap, count);
}

}  // namespace mfa
