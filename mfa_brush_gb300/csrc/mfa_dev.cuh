// mfa_dev.cuh -- device-side data layout and helpers of the GB300 MD-DPD step.
//
// Layout in HBM (one context = R replicas sharing one parameter set):
//   * particles of all replicas live in ONE sorted order ("slots"): replica-major, then by
//     neighbour-list cell, then by tag; the order is rebuilt by a counting sort when any particle
//     moved more than skin/2 since the last rebuild (check_skin.f90:11-24 semantics);
//   * master state in slot order, FP64 structure-of-arrays: r[3][Np], v[3][Np], a[3][Np], f[3][Np];
//   * pair-kernel views, rewritten by every position update:
//       mixed: int4  {x,y,z fixed point, info}  + float4  {vx,vy,vz, tag}
//       fp64 : double4{x,y,z, info bits}        + double4 {vx,vy,vz, tag bits}
//     Fixed point: x,y use 2^32 units per box length, so an int32 difference is the minimum
//     image (fluid_fluid.f90:111-112) for free; z uses 2^30 units per channel width D.
//   * full Verlet list in column-major "ELL" form: nbr[k*Np + slot], count nn[slot].
// info word: bits 0-3 type (0-based), bit 4 mobile, bit 5 brush head, bits 6-7 profile species
// (0 brush, 1 melt, 2 particle 4, 3 none), bits 8-31 replica index.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mfa {

constexpr int MAXT = 6;
constexpr int NPAIR = MAXT * MAXT;
// per-replica accumulator slots: energies, head forces, the virial tensor of each term group and the
// kinetic tensor
enum Obs { O_VFF = 0, O_VFW, O_VWW, O_VINTRA, O_VBEND, O_VBENDM, O_VOR, O_VCOUL, O_TFLUID, O_VCOULK, O_VDIP,
           O_FH = 11,  /* 6 slots: -sum of head forces, chains 1..n_chain/2 (xyz) then the others */
           O_VIR = 17, /* NVIR groups x 9 slots: W_ab = sum of F_a r_b at slot O_VIR + 9 g + 3 a + b */
           O_KIN = O_VIR + 9 * 8, /* 9 slots: sum of m v_a v_b over the mobile particles */
           NOBS = O_KIN + 9 };
// virial groups (the terms whose forces they sum)
enum VirGroup { V_PAIR = 0, V_FENE, V_BEND, V_BENDM, V_OR, V_WALL, V_KSPACE, V_DIP, NVIR };

// status bits
constexpr unsigned ST_NLIST_OVERFLOW = 1u, ST_OUT_OF_BOX = 2u, ST_NAN = 4u;

// pair flags
constexpr int PF_LJ = 1, PF_DPD_LJ = 2, PF_DPD_OWN = 4, PF_COUL = 8;

// 32-byte aligned double quadruple (one 256-bit load on sm_100 and later)
using dbl4 = double4_32a;
__host__ __device__ inline dbl4 mk_dbl4(double x, double y, double z, double w) {
  dbl4 r;
  r.x = x; r.y = y; r.z = z; r.w = w;
  return r;
}

__host__ __device__ inline int info_type(int w) { return w & 15; }
__host__ __device__ inline bool info_mobile(int w) { return (w >> 4) & 1; }
__host__ __device__ inline bool info_head(int w) { return (w >> 5) & 1; }
__host__ __device__ inline int info_species(int w) { return (w >> 6) & 3; }
__host__ __device__ inline int info_rep(int w) { return (int)((unsigned)w >> 8); }

template <typename T>
struct PairEntry {
  T range2, eps4, sig2, shift, inv_rc;  // LJ; inv_rc = 1/sqrt(range2) for the DPD weight
  T rlist2;                             // (cut-off + skin)^2 for the neighbour list
  T dpd_rc2, inv_dpd_rc;                // own DPD cut-off (DPD_CUT_OFF)
  T qq;                                 // charge product (real-space Ewald)
  T screen2;                            // largest interaction cut-off^2 (x 1.0002 in FP32): the
                                        // pair kernel's screening threshold
  int flags;
};

// Coarse int32 -> float for screening only: the difference is shifted right by `sh` bits and
// converted with one magic add (exact for |d >> sh| < 2^22); the result times 2^sh units is off
// by at most 2^sh units, covered by the margin of PairEntry::screen2.
__device__ __forceinline__ float i2f_coarse(int d, int sh) {
  return __int_as_float(0x4B400000 + (d >> sh)) - 12582912.0f;
}

// Scalars shared by every replica (passed by value).
struct SimConst {
  int n_type;
  int thermostat_dpd, dpd_weight1, force_switch_on, poiseuille, bending, bending_melt, orientation;
  int bend_form, charged, compat_i_only, wall;
  double dt, half_dt, half_dt2;
  double mass[MAXT], inv_mass[MAXT];
  double gamma, sig;             // DPD friction and noise amplitude sqrt(2 kT gamma/dt)
  double r2min_init, r2min_time; // force switch-on ramp
  double sigma_wall[MAXT], a_wall[MAXT], a_w;
  double k_chain, inv_r_chain_2, fene_xmax;
  double k_bend, alpha_eq, k_or, alpha_or, bend_small;
  double const_force[3];
  double charge[MAXT];
  double sqrt_alpha, alpha_c, inv_sqrt_pi;
  double coul_rc2;                // own Coulomb cut-off^2 (0: inside LJ range)
  double skin_half2;              // (skin/2)^2
  double va_wall[2];              // head velocity of chains 1..n_chain/2 (the others: -va_wall)
  int move_walls;                 // WALL 1 with va_wall != 0: the wall beads' sites move too
  int hist_dim;
  // FP32 copies for the mixed-precision integrator
  float dt_f, skin_half2_f, a_w_f;
  float mass_f[MAXT], inv_mass_f[MAXT], sigma_wall_f[MAXT], a_wall_f[MAXT], cforce_f[3];
  // When every interacting type pair has the same list and screening cut-offs (a single WCA or
  // LJ range), the list builder and the pair screening compare against these instead of a table
  // lookup; pairs whose own cut-off is 0 (head-head) are then listed too and dropped later.
  // 0 = cut-offs differ.
  float rl2_uni_f, scr2_uni_f;
  // FP32 copies of the pair and bond constants: a double -> float conversion issues on the FP64
  // pipe, so the mixed kernels read these instead of converting per thread
  float sig_f, gamma_f, coul_rc2_f, sqrt_alpha_f, inv_sqrt_pi_f, alpha_c_f;
  float k_chain_f, inv_r_chain_2_f, fene_xmax_f, k_bend_f, alpha_eq_f, k_or_f, alpha_or_f, bend_small_f;
};

// Per replica (device array, read through the L1).
struct RepDesc {
  double L[3], invL[3];
  double sfx[3];        // fixed-point units per sigma
  double ufx[3];        // sigma per fixed-point unit
  float ufx_f[3];
  double inv_lc[3];     // neighbour-list grid
  float lc_f[3];        // list cell edge in sigma
  float cpu_f[3];       // list cells per 512 fixed-point units
  float zlim_f[2];      // -l_cell, D + l_cell: a particle outside is out of the channel
  int nc[3];
  int cell_off, ncell;
  int p0, n_part, n_mon_tot;
  int n_mon, n_chain, n_mon_d, n_chain_d, n_mon_e, n_chain_e, part_init_d, part_init_e;
  unsigned long long seed;
  long long s_time;
  double lz_half, v_ww, inv_n;
  double v_ffw;         // LJ energy of the fixed wall beads among themselves (WALL 1; a constant)
  double v_cself;       // Ewald self energy (a constant)
  double hist_inv_dz;
  long long Lbits[2];   // bit patterns of Lx, Ly: for positive doubles, integer order = numeric order
};

// ---------------------------------------------------------------------------------------------
// Pair noise: Philox2x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), counter (min tag, max tag), key
// pair_key(seed, step).  A pair needs two 32-bit words (two uniforms for one Box-Muller normal),
// which is exactly one 2x32 block: half the multiplies of a 4x32 block, whose other two words
// would go unused.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void philox2x32_10(uint32_t& c0, uint32_t& c1, uint32_t k) {
  const uint32_t M = 0xD256D193u, W = 0x9E3779B9u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) k += W;
    const uint32_t hi = __umulhi(M, c0), lo = M * c0;
    c0 = hi ^ k ^ c1;
    c1 = lo;
  }
}

// The step's key of a replica: the low 32 bits of the step XOR a 32-bit digest of the 64-bit
// seed (the MurmurHash3 64-bit finalizer, low half).  For one replica the keys of two steps less
// than 2^24 apart differ, and no step's round keys (key + r W, r < 10) are another step's shifted
// by whole rounds: adding r W changes the top byte, which the step does not reach.
__host__ __device__ __forceinline__ uint32_t pair_key(unsigned long long seed, long long step) {
  unsigned long long h = seed;
  h ^= h >> 33;
  h *= 0xff51afd7ed558ccdULL;
  h ^= h >> 33;
  h *= 0xc4ceb9fe1a85ec53ULL;
  h ^= h >> 33;
  return (uint32_t)h ^ (uint32_t)(unsigned long long)step;
}

// Two 23-bit uniforms of the unordered pair (ta, tb): u1 in (0,1), u2 in [0,1), exact in FP32.
__device__ __forceinline__ void pair_uniform_bits(uint32_t key, int ta, int tb, uint32_t& b1, uint32_t& b2) {
  uint32_t c0 = (uint32_t)min(ta, tb), c1 = (uint32_t)max(ta, tb);
  philox2x32_10(c0, c1, key);
  b1 = c0 >> 9;
  b2 = c1 >> 9;
}

__device__ __forceinline__ float pair_gauss_f(uint32_t key, int ta, int tb) {
  uint32_t b1, b2;
  pair_uniform_bits(key, ta, tb, b1, b2);
  // b1, b2 < 2^23: 2^23 + b is exact in FP32, so the subtraction converts without an I2F
  const float f1 = __uint_as_float(0x4B000000u | b1) - 8388608.0f;
  const float f2 = __uint_as_float(0x4B000000u | b2) - 8388608.0f;
  float u1 = (f1 + 0.5f) * (1.0f / 8388608.0f);
  float u2 = f2 * (1.0f / 8388608.0f);
  // cos(2 pi u2) with u2 folded to [-1/2, 1/2] and the hardware cosine (absolute error ~3e-7
  // on [-pi, pi]); the logarithm stays the accurate one: near u1 = 1 the hardware logarithm's
  // absolute error would be comparable to -ln(u1) itself
  const float c = __cosf(6.28318548f * (u2 >= 0.5f ? u2 - 1.f : u2));
  return sqrtf(-2.0f * logf(u1)) * c;
}

__device__ __forceinline__ double pair_gauss_d(uint32_t key, int ta, int tb) {
  uint32_t b1, b2;
  pair_uniform_bits(key, ta, tb, b1, b2);
  double u1 = ((double)b1 + 0.5) * (1.0 / 8388608.0);
  double u2 = (double)b2 * (1.0 / 8388608.0);
  return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

// ---------------------------------------------------------------------------------------------
// Conversions on the fast pipes.  On GB300 the conversion instructions (I2F, F2F, F2I) issue at
// the FP64 rate, 2 per SM per clock against 128 FP32 operations, which made them the hidden
// limiter of the pair kernel (three int->float per list entry) and of the integrator.  These
// exact replacements use integer and FP32 arithmetic only.
// ---------------------------------------------------------------------------------------------
// int32 -> float, correctly rounded: high and low 16-bit halves through the 2^23 magic numbers,
// recombined with one FFMA (hi*2^16 + lo is exact before the single rounding).
__device__ __forceinline__ float i2f_fast(int d) {
  const float hi = __int_as_float(0x4B400000 + (d >> 16)) - 12582912.0f;     // d>>16 in [-2^15, 2^15)
  const float lo = __int_as_float(0x4B000000 | (d & 0xFFFF)) - 8388608.0f;   // [0, 2^16)
  return fmaf(hi, 65536.0f, lo);
}

// float -> double, exact for normal numbers; zero and subnormals become signed zero.
__device__ __forceinline__ double f2d_fast(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu;
  const unsigned sgn = u & 0x80000000u;
  unsigned hi = sgn | ((e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3);
  unsigned lo = u << 29;
  if (e == 0) { hi = sgn; lo = 0u; }
  return __hiloint2double((int)hi, (int)lo);
}

// double -> float, round to nearest even, for |d| inside the normal float range (smaller
// magnitudes flush to signed zero; the values converted here are velocities and distances).
__device__ __forceinline__ float d2f_fast(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned hi = (unsigned)(b >> 32);
  const unsigned sgn = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7FFu) - 896;
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  unsigned mant = (unsigned)(m >> 29);
  const unsigned rem = (unsigned)(m & 0x1FFFFFFFull);
  mant += (rem > 0x10000000u || (rem == 0x10000000u && (mant & 1u))) ? 1u : 0u;
  const unsigned r = sgn | (((unsigned)e << 23) + mant);  // a mantissa carry bumps the exponent
  return __uint_as_float(e <= 0 ? sgn : r);
}

// ---------------------------------------------------------------------------------------------
// Fixed-point positions
// ---------------------------------------------------------------------------------------------
// Nearest integer (ties away from zero) of d, for |d| < 2^62, from the bit pattern: one FP64
// multiply forms d, the rounding is integer work (an FP64 magic-number add would be a second
// operation on the slow FP64 pipe).
__device__ __forceinline__ long long round_bits(double d) {
  const long long b = __double_as_longlong(d);
  const int e = (int)((b >> 52) & 0x7FF);
  const int sh = 1075 - e;                        // fractional bits of the 53-bit mantissa
  const unsigned long long m = ((unsigned long long)b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  unsigned long long r;
  if (sh <= 0) r = m << (-sh);                    // already an integer (|d| >= 2^52)
  else if (sh > 53) r = 0;                        // |d| < 1/2
  else r = (m + (1ull << (sh - 1))) >> sh;
  return (b < 0) ? -(long long)r : (long long)r;
}

__device__ __forceinline__ int to_fx_periodic(double x, double s) {
  // x in [0, L] -> [0, 2^32) modulo 2^32
  return (int)(unsigned int)(unsigned long long)round_bits(x * s);
}
__device__ __forceinline__ int to_fx_z(double z, double s) { return (int)round_bits(z * s); }
__device__ __forceinline__ int fx_diff(int a, int b) { return (int)((unsigned)a - (unsigned)b); }

// Minimum image of the reference: d - L*int(2 d / L) (fluid_fluid.f90:111-112).
__device__ __forceinline__ double mic_ref(double d, double L, double invL) {
  return d - L * (double)(long long)(2. * d * invL);
}

// ---------------------------------------------------------------------------------------------
// Reductions
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Adds v into col[rep] (one accumulator column of the slot-major [NOBS][nrep] array).  Must be called by all 32 lanes of the warp (kernels keep
// every lane alive and mask work with `active`); lanes sharing a replica are summed first, so
// the common case (one replica per warp) costs one warp reduction and one FP64 atomic.
__device__ __forceinline__ void add_obs(double* col, int rep, double v, bool active, int nrep = 0) {
  (void)nrep;
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int key = active ? rep : -1;
  unsigned todo = FULL;
  while (todo) {
    int l = __ffs(todo) - 1;
    int k = __shfl_sync(FULL, key, l);
    bool mine = (key == k);
    unsigned grp = __ballot_sync(FULL, mine);
    double s = warp_sum(mine ? v : 0.);
    if (k >= 0 && lane == l) atomicAdd(&col[k], s);
    todo &= ~grp;
  }
}

}  // namespace mfa
