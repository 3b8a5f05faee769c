// mfa_state.cuh -- device state of one context and the kernel launchers (host-callable).
#pragma once
#include "mfa_dev.cuh"

namespace mfa {

// All device pointers of a context; passed by value to kernels.
struct DevState {
  int N;       // particles (all replicas)
  int Np;      // padded stride of the neighbour list (multiple of 32)
  int nrep;
  int mixed;   // MFA_PREC_MIXED
  // master state, slot order, FP64
  double *rx, *ry, *rz, *vx, *vy, *vz, *ax, *ay, *az, *fx, *fy, *fz;
  int *tag, *info;
  // permutation scratch
  double* tmp[9];
  int *tmp_tag, *tmp_info;
  int* slot_of_tag;
  // FP32 force of the fused mixed-precision step (pair + bonded + k-space), read by the integrator
  float4* f4;
  // pair-kernel views
  int4* pfx;
  float4* vf;
  // the other view buffers of the mixed path: a pair kernel with the step's integration fused in
  // writes the next step's views there while its neighbours still read pfx and vf; the step
  // counter has a copy per buffer set for the same reason
  int4* pfx_alt;
  float4* vf_alt;
  long long* steps_alt;
  int sync_alt;  // 1: the position update that starts a chunk also copies the wall beads' views and
                 // the step counter from the other set into this one
  int permute_accel;  // 1: a rebuild carries the mobile particles' FP64 accelerations into the new
                      // order.  0 for the rebuilds inside mfa_step: there the accelerations are
                      // dead from the call's first position update to its last velocity update,
                      // which rewrites them (the wall beads' are carried either way)
  dbl4* pd;
  dbl4* vd;
  int4* ref;   // fixed-point position at the last rebuild
  // neighbour list
  int *nn, *nbr;
  int nbr_cap;
  // cells
  int *cell_of, *rank, *perm, *cell_count, *cell_start;
  int* scan_blk;              // [2 * 256] block sums and offsets of the cell-start scan
  int ncell_tot;
  // control words
  float rl2_uni;  // SimConst::rl2_uni_f (0: per-pair list cut-offs)
  int nl_h;       // list-build cells per list cut-off; the search covers (2 nl_h + 1)^3 cells
  int nl_hx;      // the same along x alone (nl_h unless list_cells_x; only with nl_h 1)
  int pair_persist;  // mfa_options.pair_schedule
  int* pair_q;       // [2] the persistent pair kernel's queue: next tile, blocks finished
  int* rebuild_flag;          // [1 + nrep]: [0] some replica needs a rebuild, [1 + r] replica r does
  int* cell_rep;              // [ncell_tot] replica of each list cell
  // work list of a rebuild (k_worklist): the replicas to rebuild in ascending order (wl_rep), the
  // prefix sums over them of their particles (wl_p), cells (wl_c) and list-builder chunks (wl_k),
  // each [nrep + 1], their number (wl_n[0]) and the list builder's chunk queue (wl_n[1])
  int *wl_rep, *wl_p, *wl_c, *wl_k, *wl_n;
  int nsm;                    // streaming multiprocessors of the device (grids of the rebuild)
  long long* rebuilds;        // [1] rebuild events (any replica)
  long long* rep_rebuilds;    // [nrep] rebuilds of each replica
  unsigned* status;
  long long* steps_done;
  // tables
  const RepDesc* reps;
  const PairEntry<float>* tabf;
  const PairEntry<double>* tabd;
};

// energy accumulators: slot-major [NOBS][nrep]
struct Acc {
  double* a;
  int nrep;
  __host__ __device__ double* col(int slot) const { return a + (size_t)slot * nrep; }
};

// Adds NV per-thread values v[c] into the accumulator columns slot[c] at the thread's replica.
// All 32 lanes of the warp must call it (inactive lanes add nothing).  When every active lane of
// the warp belongs to one replica (the common case: particles are sorted by replica), the warp
// sums all values at once by a transpose reduction in T (each of 5 exchange rounds halves the
// values a lane holds: 31 shuffles for 32 values, after which lane c holds the sum of value c) and
// lane c adds it to its column with one FP64 atomic; otherwise each value takes add_obs.
// (T = float in the mixed-precision kernels: the warp sums run on the FP32 pipe, not on the
// FP64 one, which GB300 issues at 1/64 of the FP32 rate.)
template <typename T, int NV>
__device__ __forceinline__ void obs_push(const Acc& acc, const int (&slot)[NV], const T (&v)[NV], int rep,
                                         bool active) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned act = __ballot_sync(FULL, active);
  if (!act) return;
  const int r0 = __shfl_sync(FULL, rep, __ffs(act) - 1);
  if (__all_sync(FULL, !active || rep == r0)) {
#pragma unroll
    for (int base = 0; base < NV; base += 32) {
      T u[32];
#pragma unroll
      for (int c = 0; c < 32; ++c) u[c] = (active && base + c < NV) ? v[base + c < NV ? base + c : 0] : T(0);
#pragma unroll
      for (int off = 16; off >= 1; off >>= 1) {
        const bool up = (lane & off) != 0;
#pragma unroll
        for (int j = 0; j < off; ++j) {
          const T send = up ? u[j] : u[j + off];
          const T keep = up ? u[j + off] : u[j];
          u[j] = keep + __shfl_xor_sync(FULL, send, off);
        }
      }
      int sl = -1;
#pragma unroll
      for (int c = 0; c < 32; ++c)
        if (c == lane && base + c < NV) sl = slot[base + c];
      const double t = (double)u[0];
      if (sl >= 0 && t != 0.) atomicAdd(acc.col(sl) + r0, t);
    }
  } else {
#pragma unroll
    for (int c = 0; c < NV; ++c) add_obs(acc.col(slot[c]), rep, (double)v[c], active, acc.nrep);
  }
}

// A symmetric tensor into the 9 slots from `base` (a virial group O_VIR + 9 g, or O_KIN): six
// components xx yy zz xy xz yz, the host mirrors them to yx zx zy.  One add_obs per component, so
// all 32 lanes of the warp must call it.
template <typename T>
__device__ __forceinline__ void add_obs_sym(const Acc& acc, int base, int rep, const T* w6, bool active) {
  const int idx[6] = {0, 4, 8, 1, 2, 5};
#pragma unroll
  for (int c = 0; c < 6; ++c) add_obs(acc.col(base + idx[c]), rep, (double)w6[c], active, acc.nrep);
}
// A general tensor (9 components, row-major a b).
template <typename T>
__device__ __forceinline__ void add_obs9(const Acc& acc, int base, int rep, const T* w9, bool active) {
#pragma unroll
  for (int c = 0; c < 9; ++c) add_obs(acc.col(base + c), rep, (double)w9[c], active, acc.nrep);
}
// w6 += c d (x) d (symmetric, xx yy zz xy xz yz)
template <typename T>
__device__ __forceinline__ void sym_add(T* w6, T c, T dx, T dy, T dz) {
  const T cx = c * dx, cy = c * dy;
  w6[0] += cx * dx; w6[1] += cy * dy; w6[2] += c * dz * dz;
  w6[3] += cx * dy; w6[4] += cx * dz; w6[5] += cy * dz;
}

// ---- rebuild (cell sort + neighbour list) --------------------------------------------------------
// Rebuilds the replicas whose flag is set (every replica when `force`), then counts the rebuild
// and clears the flags.
void launch_rebuild(const DevState& s, cudaStream_t st, bool force);
// The skin test's outcome for replica `rep` (check_skin.f90:11-24 decides per system).
__device__ __forceinline__ void flag_rebuild(const DevState& s, int rep) {
  s.rebuild_flag[1 + rep] = 1;
  s.rebuild_flag[0] = 1;
}
// largest neighbour-list capacity (entries per particle) a context may grow to
constexpr int NL_CAP_MAX = 420;
// ---- forces ------------------------------------------------------------------------------------
// pair forces (fluid_fluid); accumulate = add into f, else overwrite; eflag = energies into acc;
// bonded_mask != 0 in the fused mixed step (overwrite into f4) adds the bonded terms in the same
// kernel (the caller then skips launch_bonded)
// integ (the fused mixed step without energies, one block per tile): the step's integration in the
// pair kernel's tail, views to the other buffer set (k_pair's INTEG)
void launch_pair(const DevState& s, const SimConst& C, cudaStream_t st, bool accumulate, bool eflag,
                 Acc acc, int block, int bonded_mask = 0, bool integ = false);
// bonded terms: mask bit 1 FENE, 2 brush bending, 4 melt bending, 8 orientation
void launch_bonded(const DevState& s, const SimConst& C, cudaStream_t st, int mask, bool eflag, Acc acc,
                   bool fused = false);
// implicit 9-3 walls (fluid_wall 2) and constant body force (constant_force 1)
void launch_wall(const DevState& s, const SimConst& C, cudaStream_t st, bool eflag, Acc acc);
void launch_const_force(const DevState& s, const SimConst& C, cudaStream_t st);
// ---- integration -------------------------------------------------------------------------------
// mode 0: verlet_positions; 1: verlet_velocities; 2: velocities(n) + positions(n+1) fused.
// add_ext: add the 9-3 wall and constant body forces inside the kernel (fused path).
void launch_integrate(const DevState& s, const SimConst& C, cudaStream_t st, int mode, bool add_ext,
                      bool eflag, Acc acc);
void launch_profiles(const DevState& s, const SimConst& C, cudaStream_t st, double* prof, int hist);
void launch_record(Acc acc, double* out, cudaStream_t st);
// observation quantities per replica: out[9 r + 0..2] brush Rg^2, 3..5 melt Rg^2, 6..8 momentum
void launch_observe(const DevState& s, const SimConst& C, cudaStream_t st, double* out);
// one observation into the averages avg[nrep][NAVG] (mfa_obs.cuh) from the record and out above
void launch_obs_accum(const DevState& s, const SimConst& C, cudaStream_t st, const double* rec, const double* obs,
                      double* avg);
// the record's energy slots into the series ring [cap][O_VIR][nrep] at *head, then ++*head
void launch_series(const DevState& s, cudaStream_t st, const double* rec, double* series, long long* series_step,
                   long long* head, int cap);
// ---- host <-> device layout ----------------------------------------------------------------------
// canonical AoS (3*tag+d) <-> slot order
void launch_scatter_state(const DevState& s, cudaStream_t st, const double* r, const double* v,
                          const double* a);
void launch_gather_state(const DevState& s, cudaStream_t st, double* r, double* v, double* a, double* f);
void launch_init_views(const DevState& s, cudaStream_t st);
// views from the current r, v plus the skin test against the last rebuild (sets rebuild_flag)
void launch_refresh_views(const DevState& s, const SimConst& C, cudaStream_t st);
// ---- parity exports ----------------------------------------------------------------------------
void launch_ref_cells(const DevState& s, cudaStream_t st, int rep, const double* inv_l, const int* nc,
                      int* cell_of_tag, int* counts);
void launch_cell_neigh(const int* nc, int n_nei, int* out, cudaStream_t st);
void launch_pair_list(const DevState& s, const SimConst& C, cudaStream_t st, int rep, int* pairs,
                      long long cap, unsigned long long* count);
// ---- k-space Ewald (ewald_k.f90, dipolar_correction.f90) ------------------------------------
// exp(i k.r) = X(nx) Y(ny) Z(nz) per charged particle: the tables hold X for nx = 0..nxm,
// Y for ny = 0..nym and Z for nz = 0..nzm (negative n by conjugation).
// The k-vectors come in the reference's order: kz outer, ky, kx inner, so every (ky, kz) pair
// owns one contiguous run of k ("row") whose phases share the factor Y Z: a (k, particle) term
// then costs one complex product instead of a sin/cos of a large argument.
struct KSpace {
  int nk, nq, nxm, nym, nzm, ncol;
  int4* kn;             // [nk] (nx, ny, nz, 0) in the reference's enumeration order
  double* kvec;         // [3*nk]
  double* kfac;         // [nk] exp(-k^2/(4 alpha_c)) / k^2
  float2* tabf;         // [ncol][nq] (mixed): X(0..nxm), Y(0..nym), Z(0..nzm) per particle
  double2* tabd;        // [ncol][nq] (fp64)
  int* qtag;            // [nq] tags of the charged particles
  double* qval;         // [nq] their charges
  float* qvalf;         // [nq] the same in FP32
  double cx, cy, cz;    // dk/(2 pi) per axis
  double inv_V, lz_half;
  double* mz;           // [1] dipole moment M_z
  // rows
  int nrows;
  int4* rows;           // [nrows] (first k, end k, ny, nz)
  int* krow;            // [nk] row of each k
  // rho: blocks of rows and nx slots x particle chunks; partials summed in a fixed order.
  // The dense slot table has 4 qx slots per row, nx = -nxm .. -nxm + 4 qx - 1.
  int qx;
  int pchunk, npchunks;
  double* rho_part;     // [npchunks][2*nk]
  float4* kdf;          // [nk] (kx, G Re rho, G Im rho, nx + nxm as int bits)   (mixed)
  double2* kdd;         // [nk] (G Re rho, G Im rho)                              (fp64)
  float4* wdense;       // [nrows][4 qx] (W, kx W) per slot, W = G rho, rows in frow order;
                        // zero where no k (mixed)
  int* frow;            // [nrows] rows in order of their slot range (force order) ...
  int* fpos;            // [nrows] ... and the position of each row in that order
  int2* fwin;           // [nkchunks] slot window of each force chunk (dense kernel)
  // force: chunks of KS_FR whole rows
  int nkchunks, fchunk_k_max, fchunk_rows_max;
  int* chunk_row;       // [nkchunks+1] first row of each chunk
  double* fpart;        // [nkchunks][nq][3] per-chunk force partials, summed in a fixed order
  // deterministic grid reductions: per-block partials, the last block to finish sums them
  double* red_part;     // [8*KS_RED_MAX]: rho_sum energy and virial (7 per block), dipole moment
  unsigned* ticket;     // [2] zero between launches
  int rep;
  int plain;            // 1: FP32 sums without Kahan compensation (mfa_options.kspace_plain_sums)
};
constexpr int KS_FB = 128;       // particles per force block
constexpr int KS_FR = 32;        // rows per force chunk
constexpr int KS_RED_MAX = 256;  // blocks of a grid reduction, at most
constexpr size_t KS_SMEM_MAX = 227 * 1024;  // dynamic shared memory of one block, at most
// the dense force kernel (X in registers) serves mixed precision with nxm <= 15
bool kspace_dense(const KSpace& K, bool mixed);
// shared memory of the one-k-at-a-time force kernel for the chunks set in K
size_t kspace_force_smem(const KSpace& K, bool mixed);
// host-side preparation of the kernels (shared-memory opt-in); returns a CUDA error
int kspace_prepare(const KSpace& K, bool mixed);
// fused: the mixed-precision fused step adds into the FP32 force array, otherwise into FP64
void launch_kspace(const DevState& s, const SimConst& C, const KSpace& K, cudaStream_t st, bool eflag, Acc acc,
                   bool fused = false);
void launch_dipolar(const DevState& s, const SimConst& C, const KSpace& K, cudaStream_t st, bool eflag, Acc acc,
                    bool fused = false);

// implicit 9-3 walls (fluid_wall.f90:93-121): the bottom wall's F_z in fb, the top wall's in ft,
// e = energy of both walls
__device__ __forceinline__ void wall93_split(const SimConst& C, int t, double z, double D, double& fb, double& ft,
                                             double& e) {
  const double sw = C.sigma_wall[t], awt = C.a_wall[t], aw = fabs(awt);
  const double sw3 = sw * sw * sw, sw9 = sw3 * sw3 * sw3;
  double iz = 1. / z;
  double iz2 = iz * iz, iz4 = iz2 * iz2, iz8 = iz4 * iz4, iz10 = iz8 * iz2;
  double rd = sw * iz, rd3 = rd * rd * rd, rd9 = rd3 * rd3 * rd3;
  e = aw * rd9 - C.a_w * rd3;
  fb = 9. * aw * sw9 * iz10;
  fb -= 3. * awt * sw3 * iz4;
  iz = 1. / (D - z);
  iz2 = iz * iz; iz4 = iz2 * iz2; iz8 = iz4 * iz4; iz10 = iz8 * iz2;
  rd = sw * iz; rd3 = rd * rd * rd; rd9 = rd3 * rd3 * rd3;
  e += aw * rd9 - C.a_w * rd3;
  ft = -9. * aw * sw9 * iz10;
  ft += 3. * awt * sw3 * iz4;
}

__device__ __forceinline__ double wall93(const SimConst& C, int t, double z, double D, double& e) {
  double fb, ft;
  wall93_split(C, t, z, D, fb, ft, e);
  return fb + ft;
}

// The same in FP32 from the distances to the bottom (zl) and top (zh) wall; 9|A| s^9 z^-10 =
// 9|A| (s/z)^9 / z, 3 A s^3 z^-4 = 3 A (s/z)^3 / z.
__device__ __forceinline__ void wall93f_split(const SimConst& C, int t, float zl, float zh, float& fb, float& ft,
                                              float& e) {
  const float sw = C.sigma_wall_f[t], awt = C.a_wall_f[t], aw = fabsf(awt), a_w = C.a_w_f;
  float iz = 1.f / zl, rd = sw * iz, rd3 = rd * rd * rd, rd9 = rd3 * rd3 * rd3;
  e = aw * rd9 - a_w * rd3;
  fb = (9.f * aw * rd9 - 3.f * awt * rd3) * iz;
  iz = 1.f / zh; rd = sw * iz; rd3 = rd * rd * rd; rd9 = rd3 * rd3 * rd3;
  e += aw * rd9 - a_w * rd3;
  ft = -(9.f * aw * rd9 - 3.f * awt * rd3) * iz;
}

}  // namespace mfa
