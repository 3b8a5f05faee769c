// mfa_kspace.cu -- reciprocal-space Ewald sum with the slab correction on the device.
//
// ewald_k.f90:128-202 evaluates rho(k) = sum_i q_i exp(i k.r_i) over N_k half-space vectors and
// then F_i = -(8 pi q_i / V) sum_k k G(k) (cos(k.r_i) Im rho - sin(k.r_i) Re rho),
// U = (4 pi / V) sum_k G(k) |rho(k)|^2, G(k) = exp(-k^2/(4 alpha_c)) / k^2, storing an N x N_k
// phase array.  Here nothing of size N x N_k is stored.  The k-vectors come kz outer, ky, kx
// inner, so a (ky, kz) "row" of k shares the factor Y(ky) Z(kz) and only X(kx) varies along it:
//   k_ks_tables:  per charged particle, X(nx) = exp(i nx dkx x), Y(ny), Z(nz) for n >= 0, each
//                 from an FP64 phase reduced to [-1/2, 1/2) turns (sincospi); stored column-major
//                 ([column][particle]) so that a warp reads 32 particles of one column at once;
//   k_ks_rho:     rho(row, nx) = sum_p (q Y Z)(p, row) X(p, nx) as a complex matrix product per
//                 block of 64 rows x 16 |nx| slots x a particle chunk, +nx and -nx from the same
//                 four real sums (X(-n) = conj X(n)): lane = slot, half-warp = 4 rows, tiles of
//                 32 particles in shared memory; plain sums over a tile and Kahan-compensated
//                 sums across tiles in FP32 (MIXED), or FP64 sums; one partial per particle
//                 chunk;
//   k_ks_rho_sum: the partials of each k summed in a fixed order; G rho per k and the dense
//                 (row, slot) table of (G rho, kx G rho) for the force; U reduced
//                 deterministically (per-block partials, the last block adds them);
//   k_ks_force_dense (mixed, nxm <= 15): thread per particle with X(0..nxm) in registers, a
//                 chunk of 32 rows per block streamed from the dense table with its +nx and -nx
//                 slots folded together: per row S = sum conj(X) G rho and
//                 S_x = sum conj(X) kx G rho, then Im(conj(Y Z) S_x) to F_x and ky, kz times
//                 Im(conj(Y Z) S) to F_y, F_z; rows added with Kahan compensation;
//   k_ks_force:   the same per row, one k at a time from shared memory (FP64, or nxm > 15);
//   k_ks_force_sum: the chunk partials in a fixed order, times -8 pi q / V, into the force array.
// dipolar_correction.f90:20-33 (Yeh-Berkowitz slab term) is k_ks_dipole + k_ks_dipole_force, FP64.
// Every sum has a fixed order, so a charged run is reproducible bit for bit.
#include <type_traits>

#include "mfa_state.cuh"

namespace mfa {

template <bool MIXED>
using kreal = typename std::conditional<MIXED, float, double>::type;
template <bool MIXED>
using kcplx = typename std::conditional<MIXED, float2, double2>::type;

__device__ __forceinline__ void cmul(float2 a, float2 b, float2& c) {
  c = make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ void cmul(double2 a, double2 b, double2& c) {
  c = make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// s += y: Kahan-compensated in FP32 (c carries the negated lost low part) unless `plain` (the
// precision study of mfa_options.kspace_plain_sums), plain in FP64
template <bool MIXED>
__device__ __forceinline__ void ksum(kreal<MIXED>& s, kreal<MIXED>& c, kreal<MIXED> y, bool plain = false) {
  if constexpr (MIXED) {
    if (plain) {
      s += y;
      return;
    }
    const float z = y - c;
    const float t = s + z;
    c = (t - s) - z;
    s = t;
  } else {
    s += y;
  }
}

template <bool MIXED>
__device__ __forceinline__ const kcplx<MIXED>* ktab(const KSpace& K) {
  if constexpr (MIXED) return K.tabf; else return K.tabd;
}

template <bool MIXED>
__global__ void k_ks_tables(DevState s, KSpace K) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= K.nq * K.ncol) return;
  const int col = idx / K.nq, p = idx - col * K.nq;
  const int i = s.slot_of_tag[K.qtag[p]];
  double u;
  if (col <= K.nxm) u = (double)col * K.cx * s.rx[i];
  else if (col <= K.nxm + 1 + K.nym) u = (double)(col - K.nxm - 1) * K.cy * s.ry[i];
  else u = (double)(col - K.nxm - K.nym - 2) * K.cz * s.rz[i];
  u -= rint(u);  // turns in [-1/2, 1/2]
  if constexpr (MIXED) {
    float sn, cs;
    sincospif(2.f * (float)u, &sn, &cs);
    K.tabf[idx] = make_float2(cs, sn);
  } else {
    double sn, cs;
    sincospi(2. * u, &sn, &cs);
    K.tabd[idx] = make_double2(cs, sn);
  }
}

constexpr int KS_TILE = 32;  // particles per shared-memory tile of k_ks_rho (one per lane)

// rho(row, nx) = sum_p A(p, row) X(p, nx), A = q Y(ny) Z(nz), with X(p, -n) = conj X(p, n): the
// four real sums P1 = sum a c, P2 = sum b d, P3 = sum a d, P4 = sum b c over A = a + ib,
// X(p, n) = c + id give both rho(row, n) = (P1 - P2, P3 + P4) and rho(row, -n) = (P1 + P2,
// P4 - P3).  A block takes KS_RB rows, 16 slots n = 16 z .. 16 z + 15 (blockIdx.z) and a chunk of
// particles.  Lane l owns slot n = 16 z + (l & 15); warp w owns rows 8 w .. 8 w + 7, four of them
// per half-warp (l >> 4).  Per particle a lane reads its X (the half-warps share the 16 slots)
// and its four A (two 16-byte loads, one address per half-warp) for 16 FMAs, which cover up to
// eight k: half the products of a slot per signed nx.  Slots outside a row's k-range are
// computed and not stored.  The staging stores, one particle per lane, use odd (X) or 4 mod 32
// word (A) row strides.
constexpr int KS_RHO_T = 256;  // threads of a k_ks_rho block (8 warps)
constexpr int KS_RW = 8;       // rows per warp (four per half-warp)
constexpr int KS_RB = 64;      // rows per block
constexpr int KS_SL = 16;      // |nx| slots per block
constexpr int KS_XS = KS_SL + 1;  // X row stride (8-byte slots)
constexpr int KS_AS = KS_RB + 2;  // A row stride (8-byte slots; 16-byte aligned rows)
static_assert(KS_TILE * KS_XS * sizeof(float2) % 16 == 0, "the A rows follow the X rows 16-byte aligned");

template <bool MIXED>
__global__ void __launch_bounds__(KS_RHO_T, MIXED ? 3 : 1) k_ks_rho(KSpace K) {
  using real = kreal<MIXED>;
  using Cx = kcplx<MIXED>;
  extern __shared__ __align__(16) unsigned char shraw[];
  Cx* Xs = reinterpret_cast<Cx*>(shraw);              // [KS_TILE][KS_XS]
  Cx* As = Xs + KS_TILE * KS_XS;                      // [KS_TILE][KS_AS] (16-byte aligned: 32 x 17 x 8 B)
  int2* rc = reinterpret_cast<int2*>(As + KS_TILE * KS_AS);  // [KS_RB] signed Y column, Z column
  const Cx* tab = ktab<MIXED>(K);
  const int rbeg = blockIdx.x * KS_RB, nr = min(KS_RB, K.nrows - rbeg);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, half = lane >> 4;
  constexpr int NW = KS_RHO_T / 32;
  constexpr int RL = KS_RW / 2;  // rows per lane
  const int slot = blockIdx.z * KS_SL + (lane & (KS_SL - 1));  // |nx| of the lane
  const int r0 = warp * KS_RW + half * RL;                      // the lane's first row
  const bool act = r0 < nr;
  for (int r = threadIdx.x; r < nr; r += KS_RHO_T) {
    const int4 R = K.rows[rbeg + r];
    const int yc = K.nxm + 1 + abs(R.z);
    rc[r] = make_int2(R.z < 0 ? -yc : yc, K.nxm + K.nym + 2 + R.w);
  }
  const int p_beg = blockIdx.y * K.pchunk, p_end = min(K.nq, p_beg + K.pchunk);
  real s[4][RL], c[4][RL];  // sums P1..P4 across tiles and their compensations
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int i = 0; i < RL; ++i) s[a][i] = c[a][i] = 0;
  for (int t0 = p_beg; t0 < p_end; t0 += KS_TILE) {
    const int nt = min(KS_TILE, p_end - t0);
    __syncthreads();
    if (lane < nt) {
      const int pq = t0 + lane;
      real q;
      if constexpr (MIXED) q = K.qvalf[pq]; else q = K.qval[pq];
#pragma unroll
      for (int i = 0; i < KS_SL / NW; ++i) {  // slot columns warp + NW i
        const int n = blockIdx.z * KS_SL + warp + NW * i;
        Cx xv;
        xv.x = 0;
        xv.y = 0;
        if (n <= K.nxm) xv = tab[(size_t)n * K.nq + pq];
        Xs[lane * KS_XS + warp + NW * i] = xv;
      }
#pragma unroll
      for (int h = 0; h < KS_RB / NW; h += 4) {  // rows warp + NW (h .. h+3)
        Cx yv[4], zv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int r = warp + NW * (h + i);
          if (r < nr) {
            const int2 R = rc[r];
            yv[i] = tab[(size_t)abs(R.x) * K.nq + pq];
            zv[i] = tab[(size_t)R.y * K.nq + pq];
          }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int r = warp + NW * (h + i);
          if (r < nr) {
            if (rc[r].x < 0) yv[i].y = -yv[i].y;
            Cx A;
            cmul(yv[i], zv[i], A);
            A.x *= q;
            A.y *= q;
            As[lane * KS_AS + r] = A;
          }
        }
      }
    }
    __syncthreads();
    if (act) {
      // plain sums over the tile's particles, compensated sums across tiles
      real t[4][RL];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int i = 0; i < RL; ++i) t[a][i] = 0;
#pragma unroll 1
      for (int p = 0; p < nt; ++p) {
        const Cx x = Xs[p * KS_XS + (lane & (KS_SL - 1))];
        Cx A[RL];
        if constexpr (MIXED) {
          const float4* A4 = reinterpret_cast<const float4*>(As + p * KS_AS + r0);
#pragma unroll
          for (int i = 0; i < RL / 2; ++i) {
            const float4 u = A4[i];
            A[2 * i] = make_float2(u.x, u.y);
            A[2 * i + 1] = make_float2(u.z, u.w);
          }
        } else {
#pragma unroll
          for (int i = 0; i < RL; ++i) A[i] = As[p * KS_AS + r0 + i];
        }
#pragma unroll
        for (int i = 0; i < RL; ++i) {
          t[0][i] = fma(A[i].x, x.x, t[0][i]);
          t[1][i] = fma(A[i].y, x.y, t[1][i]);
          t[2][i] = fma(A[i].x, x.y, t[2][i]);
          t[3][i] = fma(A[i].y, x.x, t[3][i]);
        }
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int i = 0; i < RL; ++i) ksum<MIXED>(s[a][i], c[a][i], t[a][i], K.plain);
    }
  }
  if (act && slot <= K.nxm) {
    double* o = K.rho_part + (size_t)blockIdx.y * 2 * K.nk;
#pragma unroll
    for (int i = 0; i < RL; ++i) {
      const int r = r0 + i;
      if (r < nr) {
        const int4 R = K.rows[rbeg + r];
        const double p1 = (double)s[0][i] - (double)c[0][i], p2 = (double)s[1][i] - (double)c[1][i];
        const double p3 = (double)s[2][i] - (double)c[2][i], p4 = (double)s[3][i] - (double)c[3][i];
        const int lo = K.kn[R.x].x;  // the row's first nx
        const int kp = R.x + slot - lo;
        if (kp >= R.x && kp < R.y) {
          o[2 * kp] = p1 - p2;
          o[2 * kp + 1] = p3 + p4;
        }
        const int km = R.x - slot - lo;
        if (slot > 0 && km >= R.x && km < R.y) {
          o[2 * km] = p1 + p2;
          o[2 * km + 1] = p4 - p3;
        }
      }
    }
  }
}

// Block sum of v (all threads, warps in order); the same value in every thread.
__device__ __forceinline__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double b = 0.;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += red[w];
  return b;
}

// Block sum of v (all threads), then the last block of the grid to finish adds the per-block
// partials: each of its threads a strided subset in order, then a block sum; a fixed order for
// a given grid.  Returns true in thread 0 of that block, with the total in `total`.
__device__ __forceinline__ bool grid_sum_last(double v, double* part, unsigned* ticket, double& total) {
  __shared__ double red[32];
  __shared__ bool last;
  const double b = block_sum(v, red);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = b;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double t = 0.;
  for (unsigned k = threadIdx.x; k < gridDim.x; k += blockDim.x) t += ((volatile double*)part)[k];
  t = block_sum(t, red);
  if (threadIdx.x != 0) return false;
  total = t;
  *ticket = 0u;  // ready for the next launch
  return true;
}

// The same for NV values at once; part holds gridDim.x x NV partials.
template <int NV>
__device__ __forceinline__ bool grid_sum_last_n(const double* v, double* part, unsigned* ticket, double* total) {
  __shared__ double red[32];
  __shared__ bool last;
  double b[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) b[c] = block_sum(v[c], red);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int c = 0; c < NV; ++c) part[(size_t)blockIdx.x * NV + c] = b[c];
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double t[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) t[c] = 0.;
  for (unsigned k = threadIdx.x; k < gridDim.x; k += blockDim.x)
#pragma unroll
    for (int c = 0; c < NV; ++c) t[c] += ((volatile double*)part)[(size_t)k * NV + c];
#pragma unroll
  for (int c = 0; c < NV; ++c) t[c] = block_sum(t[c], red);
  if (threadIdx.x != 0) return false;
#pragma unroll
  for (int c = 0; c < NV; ++c) total[c] = t[c];
  *ticket = 0u;  // ready for the next launch
  return true;
}

// Thread (k, g) of a block of 32 k x 8 groups sums the chunk partials c = g, g + 8, ..; the
// eight group sums are then added in group order: a fixed order for every k.  With energies, the
// reciprocal-space virial sum over k of u_k (delta_ab - 2 k_a k_b (1/k^2 + 1/(4 alpha_c))) as well
// (u_k = G |rho|^2, the k's term of the energy), the derivative of the energy under a deformation
// of the cell.
template <bool MIXED>
__global__ void __launch_bounds__(256) k_ks_rho_sum(KSpace K, double pi4, double fac_alpha, Acc acc, bool eflag) {
  __shared__ double2 part[8][32];
  const int kl = threadIdx.x & 31, g = threadIdx.x >> 5;
  double u[7] = {0., 0., 0., 0., 0., 0., 0.};  // energy, then the virial xx yy zz xy xz yz
  const int nkb = (K.nk + 31) / 32;
  for (int kb = blockIdx.x; kb < nkb; kb += gridDim.x) {
    const int k = kb * 32 + kl;
    double re = 0., im = 0.;
    if (k < K.nk) {
#pragma unroll 4
      for (int c = g; c < K.npchunks; c += 8) {
        const double2 v = reinterpret_cast<const double2*>(K.rho_part + (size_t)c * 2 * K.nk)[k];
        re += v.x;
        im += v.y;
      }
    }
    part[g][kl] = make_double2(re, im);
    __syncthreads();
    if (g == 0 && k < K.nk) {
      re = 0.;
      im = 0.;
#pragma unroll
      for (int h = 0; h < 8; ++h) {
        re += part[h][kl].x;
        im += part[h][kl].y;
      }
      const double G = K.kfac[k];
      const double uk = G * (re * re + im * im);
      u[0] += uk;
      if (eflag) {
        const double kx = K.kvec[3 * k], ky = K.kvec[3 * k + 1], kz = K.kvec[3 * k + 2];
        const double c = 2. * (1. / (kx * kx + ky * ky + kz * kz) + fac_alpha) * uk;
        u[1] += uk - c * kx * kx;
        u[2] += uk - c * ky * ky;
        u[3] += uk - c * kz * kz;
        u[4] -= c * kx * ky;
        u[5] -= c * kx * kz;
        u[6] -= c * ky * kz;
      }
      if constexpr (MIXED) {
        const double kx = K.kvec[3 * k], a = G * re, b = G * im;
        const int xi = K.kn[k].x + K.nxm;
        K.kdf[k] = make_float4((float)kx, (float)a, (float)b, __int_as_float(xi));
        K.wdense[(size_t)K.fpos[K.krow[k]] * 4 * K.qx + xi] =
            make_float4((float)a, (float)b, (float)(kx * a), (float)(kx * b));
      } else {
        K.kdd[k] = make_double2(G * re, G * im);
      }
    }
    __syncthreads();
  }
  double tot[7];
  if (grid_sum_last_n<7>(u, K.red_part, K.ticket, tot) && eflag) {
    const double sc = pi4 * K.inv_V;
    acc.col(O_VCOULK)[K.rep] += tot[0] * sc;
    const int idx[6] = {0, 4, 8, 1, 2, 5};
    for (int c = 0; c < 6; ++c) acc.col(O_VIR + 9 * V_KSPACE + idx[c])[K.rep] += tot[1 + c] * sc;
  }
}

template <bool MIXED>
struct KD;
template <>
struct KD<true> {
  float kx, a, b;  // kx, G Re rho, G Im rho
  int xi;          // nx + nxm
};
template <>
struct KD<false> {
  double kx, a, b;
  int xi, pad;
};

template <bool MIXED>
__global__ void __launch_bounds__(KS_FB) k_ks_force(KSpace K) {
  using real = kreal<MIXED>;
  using Cx = kcplx<MIXED>;
  using real2 = kcplx<MIXED>;
  extern __shared__ __align__(16) unsigned char shraw[];
  const int nxc = 2 * K.nxm + 1;
  Cx* Xs = reinterpret_cast<Cx*>(shraw);                              // [nxc][KS_FB]
  KD<MIXED>* kd = reinterpret_cast<KD<MIXED>*>(Xs + nxc * KS_FB);     // [fchunk_k_max]
  int4* rs = reinterpret_cast<int4*>(kd + K.fchunk_k_max);            // [fchunk_rows_max]
  real2* ryz = reinterpret_cast<real2*>(rs + K.fchunk_rows_max);      // [fchunk_rows_max] ky, kz
  const int rb = K.chunk_row[blockIdx.y], re = K.chunk_row[blockIdx.y + 1];
  const int kb = K.rows[rb].x, ke = K.rows[re - 1].y;
  for (int k = kb + threadIdx.x; k < ke; k += KS_FB) {
    KD<MIXED> d;
    if constexpr (MIXED) {
      const float4 v = K.kdf[k];
      d.kx = v.x;
      d.a = v.y;
      d.b = v.z;
      d.xi = __float_as_int(v.w);
    } else {
      const double2 v = K.kdd[k];
      d.kx = K.kvec[3 * k];
      d.a = v.x;
      d.b = v.y;
      d.xi = K.kn[k].x + K.nxm;
      d.pad = 0;
    }
    kd[k - kb] = d;
  }
  for (int r = rb + threadIdx.x; r < re; r += KS_FB) {
    const int4 R = K.rows[r];
    const int yc = K.nxm + 1 + abs(R.z);
    rs[r - rb] = make_int4(R.x - kb, R.y - kb, R.z < 0 ? -yc : yc, K.nxm + K.nym + 2 + R.w);
    real2 w;
    w.x = (real)K.kvec[3 * R.x + 1];
    w.y = (real)K.kvec[3 * R.x + 2];
    ryz[r - rb] = w;
  }
  const Cx* tab = ktab<MIXED>(K);
  const int p = blockIdx.x * KS_FB + threadIdx.x;
  const int pc = min(p, K.nq - 1);
  for (int c = 0; c < nxc; ++c) {
    Cx v = tab[(size_t)abs(c - K.nxm) * K.nq + pc];
    if (c < K.nxm) v.y = -v.y;
    Xs[c * KS_FB + threadIdx.x] = v;
  }
  __syncthreads();
  if (p >= K.nq) return;
  const Cx* T = tab + pc;
  const Cx* X = Xs + threadIdx.x;
  real fx = 0, fy = 0, fz = 0, cx = 0, cy = 0, cz = 0;
  const int nr = re - rb;
  int4 R = rs[0];
  Cx Y = T[(size_t)abs(R.z) * K.nq], Z = T[(size_t)R.w * K.nq];
  for (int r = 0; r < nr; ++r) {
    // the next row's factors are loaded while this row is summed
    int4 Rn = R;
    Cx Yn = Y, Zn = Z;
    if (r + 1 < nr) {
      Rn = rs[r + 1];
      Yn = T[(size_t)abs(Rn.z) * K.nq];
      Zn = T[(size_t)Rn.w * K.nq];
    }
    if (R.z < 0) Y.y = -Y.y;
    Cx YZ;
    cmul(Y, Z, YZ);
    // plain sums along the row (at most 2 nxm + 1 terms), compensated sums across rows
    real srow = 0, sxrow = 0;
#pragma unroll 4
    for (int k = R.x; k < R.y; ++k) {
      const KD<MIXED> d = kd[k];
      Cx E;
      cmul(X[d.xi * KS_FB], YZ, E);
      const real sg = E.x * d.b - E.y * d.a;
      sxrow = fma(d.kx, sg, sxrow);
      srow += sg;
    }
    const real2 w = ryz[r];
    ksum<MIXED>(fx, cx, sxrow, K.plain);
    ksum<MIXED>(fy, cy, w.x * srow, K.plain);
    ksum<MIXED>(fz, cz, w.y * srow, K.plain);
    R = Rn;
    Y = Yn;
    Z = Zn;
  }
  double* o = K.fpart + ((size_t)blockIdx.y * K.nq + p) * 3;
  o[0] = (double)fx - (double)cx;
  o[1] = (double)fy - (double)cy;
  o[2] = (double)fz - (double)cz;
}

// Mixed precision, nxm <= 15: the thread keeps X(p, n) for n = 0 .. nxm in registers and reads
// the slot table of a chunk of rows from shared memory.  With S = sum_nx conj(X) W and
// Sx = sum_nx conj(X) kx W over a row (W = G rho), that row adds Im(conj(Y Z) Sx) to F_x and
// ky, kz times Im(conj(Y Z) S) to F_y, F_z.  X(p, -n) = conj X(p, n) and kx(-n) = -kx(n), so the
// two signed slots +-n fold into one: with X(n) = c + id, W(n) = u + iv, W(-n) = u' + iv',
//   S  gets c (u + u') + d (v - v') + i [c (v + v') - d (u - u')],
//   Sx gets c (ku + ku') + d (kv - kv') + i [c (kv + kv') - d (ku - ku')],
// where ku = kx(n) u, ku' = kx(-n) u' (the table's kx W columns): eight FMAs per |n| from two
// broadcast 16-byte loads, where the signed slots took sixteen.  The block folds the signed slot
// table (k_ks_rho_sum's (W, kx W) per signed slot) while staging it.  The rows are taken in order
// of their slot range (frow), so that the rows of a chunk share a narrow window of slots; slots
// outside the window are skipped (a branch uniform over the block).
template <int QF>
__global__ void __launch_bounds__(KS_FB) k_ks_force_dense(KSpace K) {
  constexpr int NF = 4 * QF;  // folded slots |n| = 0 .. NF - 1
  extern __shared__ __align__(16) unsigned char shraw[];
  float4* Wd = reinterpret_cast<float4*>(shraw);              // [KS_FR][NF][2]
  int2* rc = reinterpret_cast<int2*>(Wd + KS_FR * NF * 2);    // [KS_FR] signed Y column, Z column
  float2* ryz = reinterpret_cast<float2*>(rc + KS_FR);        // [KS_FR] ky, kz
  const int rbeg = blockIdx.y * KS_FR, nr = min(KS_FR, K.nrows - rbeg);
  const int nxm = K.nxm, nsig = 4 * K.qx;
  const int2 win = K.fwin[blockIdx.y];  // signed slots win.x .. win.y (slot j is nx = j - nxm)
  // the folded window: |nx| from mlo to mhi
  const int ax = abs(win.x - nxm), ay = abs(win.y - nxm);
  const int mlo = (win.x <= nxm && nxm <= win.y) ? 0 : min(ax, ay), mhi = max(ax, ay);
  const float4* wsrc = K.wdense + (size_t)rbeg * nsig;
  for (int e = threadIdx.x; e < nr * NF; e += KS_FB) {
    const int r = e / NF, m = e - r * NF;
    float4 wp = make_float4(0.f, 0.f, 0.f, 0.f), wm = wp;
    if (m <= nxm) {
      wp = wsrc[r * nsig + nxm + m];
      if (m > 0) wm = wsrc[r * nsig + nxm - m];
    }
    Wd[2 * e] = make_float4(wp.x + wm.x, wp.y - wm.y, wp.y + wm.y, wp.x - wm.x);
    Wd[2 * e + 1] = make_float4(wp.z + wm.z, wp.w - wm.w, wp.w + wm.w, wp.z - wm.z);
  }
  for (int r = threadIdx.x; r < nr; r += KS_FB) {
    const int4 R = K.rows[K.frow[rbeg + r]];
    const int yc = nxm + 1 + abs(R.z);
    rc[r] = make_int2(R.z < 0 ? -yc : yc, nxm + K.nym + 2 + R.w);
    ryz[r] = make_float2((float)K.kvec[3 * R.x + 1], (float)K.kvec[3 * R.x + 2]);
  }
  const int p = blockIdx.x * KS_FB + threadIdx.x;
  const int pc = min(p, K.nq - 1);
  const float2* T = K.tabf + pc;
  float2 X[NF];
#pragma unroll
  for (int j = 0; j < NF; ++j) {
    X[j] = make_float2(0.f, 0.f);
    if (j >= mlo && j <= mhi && j <= nxm) X[j] = T[(size_t)j * K.nq];
  }
  __syncthreads();
  if (p >= K.nq) return;
  float fx = 0.f, fy = 0.f, fz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
  int2 R = rc[0];
  float2 Y = T[(size_t)abs(R.x) * K.nq], Z = T[(size_t)R.y * K.nq];
  for (int r = 0; r < nr; ++r) {
    int2 Rn = R;
    float2 Yn = Y, Zn = Z;
    if (r + 1 < nr) {
      Rn = rc[r + 1];
      Yn = T[(size_t)abs(Rn.x) * K.nq];
      Zn = T[(size_t)Rn.y * K.nq];
    }
    if (R.x < 0) Y.y = -Y.y;
    float2 YZ;
    cmul(Y, Z, YZ);
    const float4* w = Wd + r * NF * 2;
    float s_re = 0.f, s_im = 0.f, x_re = 0.f, x_im = 0.f;
#pragma unroll
    for (int g = 0; g < QF; ++g) {  // groups of four slots; a group outside the window is skipped
      if (4 * g + 3 < mlo || 4 * g > mhi) continue;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float2 x = X[4 * g + i];
        const float4 a = w[2 * (4 * g + i)], b = w[2 * (4 * g + i) + 1];
        s_re = fmaf(x.x, a.x, fmaf(x.y, a.y, s_re));
        s_im = fmaf(x.x, a.z, fmaf(-x.y, a.w, s_im));
        x_re = fmaf(x.x, b.x, fmaf(x.y, b.y, x_re));
        x_im = fmaf(x.x, b.z, fmaf(-x.y, b.w, x_im));
      }
    }
    const float srow = YZ.x * s_im - YZ.y * s_re;
    const float sxrow = YZ.x * x_im - YZ.y * x_re;
    const float2 kyz = ryz[r];
    ksum<true>(fx, cx, sxrow, K.plain);
    ksum<true>(fy, cy, kyz.x * srow, K.plain);
    ksum<true>(fz, cz, kyz.y * srow, K.plain);
    R = Rn;
    Y = Yn;
    Z = Zn;
  }
  double* o = K.fpart + ((size_t)blockIdx.y * K.nq + p) * 3;
  o[0] = (double)fx - (double)cx;
  o[1] = (double)fy - (double)cy;
  o[2] = (double)fz - (double)cz;
}

// F_i = -(8 pi q_i / V) * sum over k-chunks in a fixed order, added to the FP64 force array or,
// in the fused mixed-precision step, to the FP32 one.
__global__ void k_ks_force_sum(DevState s, KSpace K, double pi8, bool to_f4) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= K.nq) return;
  double f[3] = {0., 0., 0.};
  for (int c = 0; c < K.nkchunks; ++c)
    for (int d = 0; d < 3; ++d) f[d] += K.fpart[((size_t)c * K.nq + p) * 3 + d];
  const int i = s.slot_of_tag[K.qtag[p]];
  const double qf = -pi8 * K.qval[p] * K.inv_V;
  if (to_f4) {
    float4 g = s.f4[i];
    g.x += (float)(qf * f[0]);
    g.y += (float)(qf * f[1]);
    g.z += (float)(qf * f[2]);
    s.f4[i] = g;
  } else {
    s.fx[i] += qf * f[0];
    s.fy[i] += qf * f[1];
    s.fz[i] += qf * f[2];
  }
}

namespace {
size_t rho_smem(const KSpace& K, bool mixed) {
  return (size_t)KS_TILE * (KS_XS + KS_AS) * (mixed ? sizeof(float2) : sizeof(double2)) +
         (size_t)KS_RB * sizeof(int2);
}
size_t force_smem(const KSpace& K, bool mixed) {
  const size_t cx = mixed ? sizeof(float2) : sizeof(double2);
  return (size_t)(2 * K.nxm + 1) * KS_FB * cx + (size_t)K.fchunk_k_max * (mixed ? sizeof(KD<true>) : sizeof(KD<false>)) +
         (size_t)K.fchunk_rows_max * (sizeof(int4) + cx);
}
// groups of four folded slots |nx| = 0 .. nxm of k_ks_force_dense
int dense_qf(const KSpace& K) { return (K.nxm + 4) / 4; }
size_t dense_smem(const KSpace& K) {
  return (size_t)KS_FR * (4 * dense_qf(K) * 2 * sizeof(float4) + sizeof(int2) + sizeof(float2));
}
constexpr int KS_DENSE_QX_MAX = 8;  // the register-resident X of k_ks_force_dense: nxm <= 15

template <int QF>
void launch_dense(const KSpace& K, dim3 g, cudaStream_t st) {
  k_ks_force_dense<QF><<<g, KS_FB, dense_smem(K), st>>>(K);
}
typedef void (*dense_launcher)(const KSpace&, dim3, cudaStream_t);
const dense_launcher kDense[5] = {nullptr, launch_dense<1>, launch_dense<2>, launch_dense<3>, launch_dense<4>};
bool use_dense(const KSpace& K, bool mixed) { return mixed && K.qx <= KS_DENSE_QX_MAX; }
}  // namespace

bool kspace_dense(const KSpace& K, bool mixed) { return use_dense(K, mixed); }
size_t kspace_force_smem(const KSpace& K, bool mixed) { return force_smem(K, mixed); }

int kspace_prepare(const KSpace& K, bool mixed) {
  const size_t a = rho_smem(K, mixed), b = use_dense(K, mixed) ? dense_smem(K) : force_smem(K, mixed);
  if (a > KS_SMEM_MAX || b > KS_SMEM_MAX) return (int)cudaErrorInvalidConfiguration;
  // The opt-in is a property of the kernel for the whole process, not of a context: set it to the
  // largest allowed size once, so that no context lowers it below another's needs (occupancy
  // follows the size of each launch, not this limit).
  const int mx = (int)KS_SMEM_MAX;
  cudaError_t e = cudaFuncSetAttribute(k_ks_rho<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_ks_rho<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_ks_force<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_ks_force<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  return (int)e;  // dense_smem stays below 48 KB: 32 rows x 16 folded slots x 32 B + 512 B
}

void launch_kspace(const DevState& s, const SimConst& C, const KSpace& K, cudaStream_t st, bool eflag, Acc acc,
                   bool fused) {
  if (K.nk == 0 || K.nq == 0) return;
  const double pi = (double)3.1415926536f;  // mfa_common.f90:315 (single-precision literal)
  const int nt = K.nq * K.ncol;
  if (s.mixed) k_ks_tables<true><<<(nt + 255) / 256, 256, 0, st>>>(s, K);
  else k_ks_tables<false><<<(nt + 255) / 256, 256, 0, st>>>(s, K);
  const dim3 g1((K.nrows + KS_RB - 1) / KS_RB, K.npchunks, (K.nxm + KS_SL) / KS_SL);
  const size_t shm1 = rho_smem(K, s.mixed);
  if (s.mixed) k_ks_rho<true><<<g1, KS_RHO_T, shm1, st>>>(K);
  else k_ks_rho<false><<<g1, KS_RHO_T, shm1, st>>>(K);
  const int gs = std::min(KS_RED_MAX, (K.nk + 31) / 32);
  const double fac_alpha = 1. / (4. * C.alpha_c);
  if (s.mixed) k_ks_rho_sum<true><<<gs, 256, 0, st>>>(K, 4. * pi, fac_alpha, acc, eflag);
  else k_ks_rho_sum<false><<<gs, 256, 0, st>>>(K, 4. * pi, fac_alpha, acc, eflag);
  const dim3 g2((K.nq + KS_FB - 1) / KS_FB, K.nkchunks);
  if (use_dense(K, s.mixed)) {
    kDense[dense_qf(K)](K, g2, st);
  } else {
    const size_t shm2 = force_smem(K, s.mixed);
    if (s.mixed) k_ks_force<true><<<g2, KS_FB, shm2, st>>>(K);
    else k_ks_force<false><<<g2, KS_FB, shm2, st>>>(K);
  }
  k_ks_force_sum<<<(K.nq + 127) / 128, 128, 0, st>>>(s, K, 8. * pi, fused && s.mixed);
}

__global__ void __launch_bounds__(256) k_ks_dipole(DevState s, KSpace K, double pi, Acc acc, bool eflag) {
  double m = 0.;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K.nq; p += gridDim.x * blockDim.x) {
    const int i = s.slot_of_tag[K.qtag[p]];
    m += K.qval[p] * (s.rz[i] - K.lz_half);
  }
  double tot;
  if (grid_sum_last(m, K.red_part + 7 * KS_RED_MAX, K.ticket + 1, tot)) {
    K.mz[0] = tot;
    if (eflag) acc.col(O_VDIP)[K.rep] += 2. * pi * tot * tot * K.inv_V;
  }
}

__global__ void k_ks_dipole_force(DevState s, KSpace K, double pi, bool to_f4) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= K.nq) return;
  const int i = s.slot_of_tag[K.qtag[p]];
  const double f = -4. * pi * K.qval[p] * K.mz[0] * K.inv_V;
  if (to_f4) s.f4[i].z += (float)f;
  else s.fz[i] += f;
}

void launch_dipolar(const DevState& s, const SimConst& C, const KSpace& K, cudaStream_t st, bool eflag, Acc acc,
                    bool fused) {
  (void)C;
  if (K.nq == 0) return;
  const double pi = (double)3.1415926536f;
  const int g = std::min(KS_RED_MAX, (K.nq + 255) / 256);
  k_ks_dipole<<<g, 256, 0, st>>>(s, K, pi, acc, eflag);
  k_ks_dipole_force<<<(K.nq + 255) / 256, 256, 0, st>>>(s, K, pi, fused && s.mixed);
}

}  // namespace mfa
