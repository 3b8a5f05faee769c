// mfa_kspace.cu -- reciprocal-space Ewald sum with the slab correction on the device.
//
// ewald_k.f90:128-202 evaluates rho(k) = sum_i q_i exp(i k.r_i) over N_k half-space vectors and
// then F_i = -(8 pi q_i / V) sum_k k G(k) (cos(k.r_i) Im rho - sin(k.r_i) Re rho),
// U = (4 pi / V) sum_k G(k) |rho(k)|^2, G(k) = exp(-k^2/(4 alpha_c)) / k^2, storing an N x N_k
// phase array.  Here nothing of size N x N_k is stored:
//   k_ks_tables: per charged particle, X(nx) = exp(i nx dkx x), Y(ny), Z(nz) for n >= 0, each
//                from an FP64 phase reduced to [-1/2, 1/2) turns (sincospi), so every factor is
//                accurate to the working precision;
//   k_ks_rho:    thread per k-vector, particles staged through shared memory, exp(i k.r) =
//                X Y Z (conjugated for negative n), FP32 Kahan-compensated partial sums (MIXED)
//                or FP64 sums, partials of particle chunks combined with FP64 atomics;
//   k_ks_energy: U in FP64;
//   k_ks_force:  thread per charged particle and k-chunk, the same factorised phase, forces
//                added to the FP64 force array.
// dipolar_correction.f90:20-33 (Yeh-Berkowitz slab term) is k_ks_dipole + k_ks_dipole_force, FP64.
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

template <bool MIXED>
__global__ void k_ks_tables(DevState s, KSpace K) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= K.nq * K.ncol) return;
  int p = idx / K.ncol, col = idx % K.ncol;
  int i = s.slot_of_tag[K.qtag[p]];
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

template <bool MIXED>
__device__ __forceinline__ kcplx<MIXED> phase_of(const kcplx<MIXED>* T, int nxm, int nym, int4 n) {
  using C = kcplx<MIXED>;
  C X = T[abs(n.x)];
  if (n.x < 0) X.y = -X.y;
  C Y = T[nxm + 1 + abs(n.y)];
  if (n.y < 0) Y.y = -Y.y;
  C Z = T[nxm + nym + 2 + n.z];
  C XY, E;
  cmul(X, Y, XY);
  cmul(XY, Z, E);
  return E;
}

constexpr int KS_TILE = 32;  // particles per shared-memory tile

template <bool MIXED>
__global__ void __launch_bounds__(256) k_ks_rho(DevState s, SimConst C, KSpace K, int chunk) {
  using real = kreal<MIXED>;
  using Cx = kcplx<MIXED>;
  extern __shared__ unsigned char shraw[];
  Cx* T = reinterpret_cast<Cx*>(shraw);           // [KS_TILE][ncol]
  real* q = reinterpret_cast<real*>(T + KS_TILE * K.ncol);
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const bool act = k < K.nk;
  const int4 n = act ? K.kn[k] : make_int4(0, 0, 0, 0);
  const int p_beg = blockIdx.y * chunk, p_end = min(K.nq, p_beg + chunk);
  real sr = 0, si = 0, cr = 0, ci = 0;  // Kahan sums
  const Cx* tab;
  if constexpr (MIXED) tab = K.tabf; else tab = K.tabd;
  for (int t0 = p_beg; t0 < p_end; t0 += KS_TILE) {
    const int nt = min(KS_TILE, p_end - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < nt * K.ncol; e += blockDim.x) T[e] = tab[(size_t)t0 * K.ncol + e];
    for (int e = threadIdx.x; e < nt; e += blockDim.x) {
      int i = s.slot_of_tag[K.qtag[t0 + e]];
      q[e] = (real)C.charge[info_type(s.info[i])];
    }
    __syncthreads();
    if (act) {
      for (int p = 0; p < nt; ++p) {
        Cx E = phase_of<MIXED>(T + p * K.ncol, K.nxm, K.nym, n);
        real yr = q[p] * E.x - cr;
        real tr = sr + yr;
        cr = (tr - sr) - yr;
        sr = tr;
        real yi = q[p] * E.y - ci;
        real ti = si + yi;
        ci = (ti - si) - yi;
        si = ti;
      }
    }
  }
  if (act) {
    atomicAdd(&K.rho[2 * k], (double)sr);
    atomicAdd(&K.rho[2 * k + 1], (double)si);
  }
}

__global__ void __launch_bounds__(1024) k_ks_energy(KSpace K, double pi4, Acc acc, bool eflag) {
  __shared__ double red[32];
  double u = 0.;
  for (int k = threadIdx.x; k < K.nk; k += blockDim.x) {
    double re = K.rho[2 * k], im = K.rho[2 * k + 1];
    u += K.kfac[k] * (re * re + im * im);
  }
  u = warp_sum(u);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = u;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.;
    v = warp_sum(v);
    if (threadIdx.x == 0 && eflag) acc.col(O_VCOULK)[K.rep] += v * pi4 * K.inv_V;
  }
}

template <bool MIXED>
__global__ void __launch_bounds__(128) k_ks_force(DevState s, SimConst C, KSpace K, int kchunk, double pi8) {
  using real = kreal<MIXED>;
  using Cx = kcplx<MIXED>;
  extern __shared__ unsigned char shraw[];
  int4* kn = reinterpret_cast<int4*>(shraw);                  // [kchunk]
  real* kd = reinterpret_cast<real*>(kn + kchunk);             // [kchunk][6] kx ky kz G Re Im
  const int k0 = blockIdx.y * kchunk, k1 = min(K.nk, k0 + kchunk);
  for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
    int kk = k - k0;
    kn[kk] = K.kn[k];
    kd[kk * 6 + 0] = (real)K.kvec[3 * k];
    kd[kk * 6 + 1] = (real)K.kvec[3 * k + 1];
    kd[kk * 6 + 2] = (real)K.kvec[3 * k + 2];
    kd[kk * 6 + 3] = (real)K.kfac[k];
    kd[kk * 6 + 4] = (real)K.rho[2 * k];
    kd[kk * 6 + 5] = (real)K.rho[2 * k + 1];
  }
  __syncthreads();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= K.nq) return;
  const Cx* T;
  if constexpr (MIXED) T = K.tabf + (size_t)p * K.ncol; else T = K.tabd + (size_t)p * K.ncol;
  real fx = 0, fy = 0, fz = 0, cx = 0, cy = 0, cz = 0;
  for (int kk = 0; kk < k1 - k0; ++kk) {
    Cx E = phase_of<MIXED>(T, K.nxm, K.nym, kn[kk]);
    const real sgl = kd[kk * 6 + 3] * (E.x * kd[kk * 6 + 5] - E.y * kd[kk * 6 + 4]);
    real y, t;
    y = kd[kk * 6 + 0] * sgl - cx; t = fx + y; cx = (t - fx) - y; fx = t;
    y = kd[kk * 6 + 1] * sgl - cy; t = fy + y; cy = (t - fy) - y; fy = t;
    y = kd[kk * 6 + 2] * sgl - cz; t = fz + y; cz = (t - fz) - y; fz = t;
  }
  double* o = K.fpart + ((size_t)blockIdx.y * K.nq + p) * 3;
  o[0] = (double)fx;
  o[1] = (double)fy;
  o[2] = (double)fz;
}

// F_i = -(8 pi q_i / V) * sum over k-chunks in a fixed order (deterministic), added to the FP64
// force array or, in the fused mixed-precision step, to the FP32 one.
__global__ void k_ks_force_sum(DevState s, SimConst C, KSpace K, double pi8, bool to_f4) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= K.nq) return;
  double f[3] = {0., 0., 0.};
  for (int c = 0; c < K.nkchunks; ++c)
    for (int d = 0; d < 3; ++d) f[d] += K.fpart[((size_t)c * K.nq + p) * 3 + d];
  const int i = s.slot_of_tag[K.qtag[p]];
  const double qf = -pi8 * C.charge[info_type(s.info[i])] * K.inv_V;
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

void launch_kspace(const DevState& s, const SimConst& C, const KSpace& K, cudaStream_t st, bool eflag, Acc acc,
                   bool fused) {
  if (K.nk == 0 || K.nq == 0) return;
  const double pi = (double)3.1415926536f;  // mfa_common.f90:315 (single-precision literal)
  int nt = K.nq * K.ncol;
  if (s.mixed) k_ks_tables<true><<<(nt + 255) / 256, 256, 0, st>>>(s, K);
  else k_ks_tables<false><<<(nt + 255) / 256, 256, 0, st>>>(s, K);
  cudaMemsetAsync(K.rho, 0, sizeof(double) * 2 * K.nk, st);
  const int kb = (K.nk + 255) / 256;
  int pchunks = max(1, min(64, (2 * 152 + kb - 1) / kb));
  int chunk = (K.nq + pchunks - 1) / pchunks;
  chunk = ((chunk + KS_TILE - 1) / KS_TILE) * KS_TILE;
  pchunks = (K.nq + chunk - 1) / chunk;
  size_t esz = s.mixed ? sizeof(float2) : sizeof(double2), rsz = s.mixed ? sizeof(float) : sizeof(double);
  size_t shm = KS_TILE * K.ncol * esz + KS_TILE * rsz;
  dim3 g1(kb, pchunks);
  if (s.mixed) k_ks_rho<true><<<g1, 256, shm, st>>>(s, C, K, chunk);
  else k_ks_rho<false><<<g1, 256, shm, st>>>(s, C, K, chunk);
  k_ks_energy<<<1, 1024, 0, st>>>(K, 4. * pi, acc, eflag);
  dim3 g2((K.nq + 127) / 128, K.nkchunks);
  size_t shm2 = K.kchunk * sizeof(int4) + K.kchunk * 6 * rsz;
  if (s.mixed) k_ks_force<true><<<g2, 128, shm2, st>>>(s, C, K, K.kchunk, 8. * pi);
  else k_ks_force<false><<<g2, 128, shm2, st>>>(s, C, K, K.kchunk, 8. * pi);
  k_ks_force_sum<<<(K.nq + 127) / 128, 128, 0, st>>>(s, C, K, 8. * pi, fused && s.mixed);
}

__global__ void __launch_bounds__(1024) k_ks_dipole(DevState s, SimConst C, KSpace K, double pi, Acc acc, bool eflag) {
  __shared__ double red[32];
  double m = 0.;
  for (int p = threadIdx.x; p < K.nq; p += blockDim.x) {
    int i = s.slot_of_tag[K.qtag[p]];
    m += C.charge[info_type(s.info[i])] * (s.rz[i] - K.lz_half);
  }
  m = warp_sum(m);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.;
    v = warp_sum(v);
    if (threadIdx.x == 0) {
      K.mz[0] = v;
      if (eflag) acc.col(O_VDIP)[K.rep] += 2. * pi * v * v * K.inv_V;
    }
  }
}

__global__ void k_ks_dipole_force(DevState s, SimConst C, KSpace K, double pi, bool to_f4) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= K.nq) return;
  int i = s.slot_of_tag[K.qtag[p]];
  const double f = -4. * pi * C.charge[info_type(s.info[i])] * K.mz[0] * K.inv_V;
  if (to_f4) s.f4[i].z += (float)f;
  else s.fz[i] += f;
}

void launch_dipolar(const DevState& s, const SimConst& C, const KSpace& K, cudaStream_t st, bool eflag, Acc acc,
                    bool fused) {
  if (K.nq == 0) return;
  const double pi = (double)3.1415926536f;
  k_ks_dipole<<<1, 1024, 0, st>>>(s, C, K, pi, acc, eflag);
  k_ks_dipole_force<<<(K.nq + 255) / 256, 256, 0, st>>>(s, C, K, pi, fused && s.mixed);
}

}  // namespace mfa
