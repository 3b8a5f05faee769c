// mfa_rebuild.cu -- cell sort and Verlet-list rebuild on the device.
//
// Replaces the reference's neighbour bookkeeping: the linked cells of cell_list.f90:56-268
// (BIN_TYPE 2, rebuilt incrementally every step) and the skin-based Verlet lists of
// binning.f90 / check_skin.f90 (BIN_TYPE 0, rebuilt when a particle moved > skin/2).  Here the
// list is rebuilt when the position kernel has raised `rebuild_flag` (displacement > skin/2):
//   1. bin:      cell of every particle on the replica's list grid (cell edge >= r_cut_max+skin),
//                per-cell counts with one atomic per particle;
//   2. scan:     cell starts from the counts of the rebuilt replicas' cells (three kernels);
//   3. place:    particle -> (cell start + atomic rank);
//   4. order:    each cell's segment sorted by tag (cells hold a handful of particles), so the
//                final order (replica, cell, tag) and every later FP sum order are deterministic;
//   5. permute:  FP64 state gathered into the new order, views and rebuild references rewritten;
//   6. list:     full neighbour list over the 27 surrounding cells (x,y periodic, z bounded).
// The decision is per replica, as the reference decides per system: the position kernel raises the
// flag of the replica whose particle moved.  k_worklist lists the flagged replicas with prefix sums
// of their particles, cells and list chunks, and every kernel after it strides over that work on a
// grid of fixed size; the other replicas' slots, cells and lists stay as they are (a replica's
// slots are one fixed range, its cells one fixed range, and its lists name only its own slots).
// In a captured CUDA graph the sequence sits in the body of a conditional node that runs only on
// steps where some replica is flagged.
#include <algorithm>

#include "mfa_state.cuh"

namespace mfa {


__device__ __forceinline__ void cell_coords(const RepDesc& R, double x, double y, double z, int& ix, int& iy,
                                            int& iz) {
  ix = (int)(x * R.inv_lc[0]);
  iy = (int)(y * R.inv_lc[1]);
  iz = (int)(z * R.inv_lc[2]);
  ix = min(max(ix, 0), R.nc[0] - 1);
  iy = min(max(iy, 0), R.nc[1] - 1);
  iz = min(max(iz, 0), R.nc[2] - 1);
}

// ---- work list ------------------------------------------------------------------------------
// The kernels of a rebuild stride over the work of the listed replicas only (their particles,
// cells or list-builder chunks) on grids of a fixed size, so a rebuild of a few replicas costs
// little more than their own work.
constexpr int WL_THREADS = 1024;
// particles per block of the list builder (one chunk of a replica's slots)
constexpr int NL_BLOCK = 128;

// The replicas to rebuild (flagged, or all when forced) and the prefix sums of their particles,
// cells and list chunks: one block, a scan over the replicas in chunks of its threads.
__global__ void __launch_bounds__(WL_THREADS) k_worklist(DevState s, bool force) {
  __shared__ int sc[4][WL_THREADS / 32];
  __shared__ int carry[4];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const bool any = force || s.rebuild_flag[0] != 0;
  if (threadIdx.x < 4) carry[threadIdx.x] = 0;
  __syncthreads();
  for (int base = 0; base < s.nrep && any; base += WL_THREADS) {
    const int r = base + threadIdx.x;
    const bool sel = r < s.nrep && (force || s.rebuild_flag[1 + r] != 0);
    int v[4] = {0, 0, 0, 0};
    if (sel) {
      const RepDesc& R = s.reps[r];
      v[0] = 1; v[1] = R.n_part; v[2] = R.ncell; v[3] = (R.n_part + NL_BLOCK - 1) / NL_BLOCK;
    }
    int x[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {  // inclusive warp scans
      x[q] = v[q];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x[q], o);
        if (lane >= o) x[q] += y;
      }
      if (lane == 31) sc[q][wid] = x[q];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int t = sc[q][lane];
        int u = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, u, o);
          if (lane >= o) u += y;
        }
        sc[q][lane] = u - t;  // exclusive warp offsets
      }
    }
    __syncthreads();
    int ex[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) ex[q] = carry[q] + sc[q][wid] + x[q] - v[q];
    if (sel) {
      s.wl_rep[ex[0]] = r;
      s.wl_p[ex[0]] = ex[1];
      s.wl_c[ex[0]] = ex[2];
      s.wl_k[ex[0]] = ex[3];
    }
    __syncthreads();
    if (threadIdx.x == WL_THREADS - 1 || r == s.nrep - 1)
#pragma unroll
      for (int q = 0; q < 4; ++q) carry[q] = ex[q] + v[q];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int n = any ? carry[0] : 0;
    s.wl_n[0] = n;
    s.wl_n[1] = 0;  // the list builder's chunk queue
    s.cell_start[s.ncell_tot] = s.N;  // the end of the last cell
    s.wl_p[n] = any ? carry[1] : 0;
    s.wl_c[n] = any ? carry[2] : 0;
    s.wl_k[n] = any ? carry[3] : 0;
  }
}

// Work item g of a prefix array pre (n listed replicas) -> its replica r and index loc inside it:
// the last k with pre[k] <= g, found by a binary search.
__device__ __forceinline__ int wl_find(const int* __restrict__ pre, int n, int g) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&pre[mid]) <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}
__device__ __forceinline__ void wl_map(const int* __restrict__ pre, const int* __restrict__ list, int n, int g,
                                       int& r, int& loc) {
  const int k = wl_find(pre, n, g);
  r = __ldg(&list[k]);
  loc = g - __ldg(&pre[k]);
}
// The same for the lanes of a warp that hold consecutive items (a grid-stride loop): the first
// active lane searches, the others step forward from its replica.
__device__ __forceinline__ int wl_map_warp(const int* __restrict__ pre, const int* __restrict__ list, int n, int g,
                                           int& r, int& loc) {
  const unsigned m = __activemask();
  const int leader = __ffs(m) - 1;
  int k = 0;
  if ((int)(threadIdx.x & 31) == leader) k = wl_find(pre, n, g);
  k = __shfl_sync(m, k, leader);
  while (k + 1 < n && __ldg(&pre[k + 1]) <= g) ++k;
  r = __ldg(&list[k]);
  loc = g - __ldg(&pre[k]);
  return k;  // the position in the list
}

#define WL_FOR(pre, g)                                                                             \
  const int wl_cnt_ = *s.wl_n;                                                                     \
  const int wl_tot_ = s.pre[wl_cnt_];                                                              \
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < wl_tot_; g += gridDim.x * blockDim.x)

__global__ void k_bin(DevState s) {
  WL_FOR(wl_p, g) {
  int rr, loc;
  wl_map_warp(s.wl_p, s.wl_rep, wl_cnt_, g, rr, loc);
  const int i = s.reps[rr].p0 + loc;
  int w = s.info[i];
  const RepDesc& R = s.reps[info_rep(w)];
  int ix, iy, iz;
  if (s.mixed) {  // the list builder's integer formula on the fixed-point view
    // (x, y need no check: the fixed-point view wraps them; the integrator flags NaN); the z
    // check in FP32, as FP64 compares and the cell-height division issue on the FP64 pipe
    const double zd = s.rz[i];
    const float z = d2f_fast(zd);
    if (!(z >= R.zlim_f[0] && z <= R.zlim_f[1]))  // also false for NaN
      atomicOr(s.status, (__double_as_longlong(zd) & 0x7FF0000000000000ll) == 0x7FF0000000000000ll ? ST_NAN
                                                                                                : ST_OUT_OF_BOX);
    const int4 q = s.pfx[i];
    ix = (int)(((unsigned long long)(unsigned)q.x * (unsigned)R.nc[0]) >> 32);
    iy = (int)(((unsigned long long)(unsigned)q.y * (unsigned)R.nc[1]) >> 32);
    iz = (int)(((long long)q.z * R.nc[2]) >> 30);
    iz = min(max(iz, 0), R.nc[2] - 1);
  } else {
    const double lz = 1. / R.inv_lc[2];
    double x = s.rx[i], y = s.ry[i], z = s.rz[i];
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) {
      atomicOr(s.status, ST_NAN);
      x = y = z = 0.;
    }
    if (z < -lz || z > R.L[2] + lz) atomicOr(s.status, ST_OUT_OF_BOX);
    cell_coords(R, x, y, z, ix, iy, iz);
  }
  const int c = R.cell_off + (iz * R.nc[1] + iy) * R.nc[0] + ix;
  s.cell_of[i] = c;
  // Particles are still nearly sorted by cell, so neighbouring lanes share cells: the lanes of one
  // cell take consecutive ranks from a single atomicAdd (k_sort_cells orders each cell by tag
  // afterwards, so the order of the ranks does not matter).
  const unsigned grp = __match_any_sync(__activemask(), c);  // the lanes still here
  const int lane = threadIdx.x & 31, leader = __ffs(grp) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(&s.cell_count[c], __popc(grp));
  base = __shfl_sync(grp, base, leader);
  s.rank[i] = base + __popc(grp & ((1u << lane) - 1u));
  }
}

// ---- cell starts of the listed replicas ---------------------------------------------------------
// The cells of the listed replicas, one after another in list order, form one sequence g; E[g] is
// the exclusive prefix sum of their counts.  A replica's counts sum to its particle count, so E at
// the first cell of the k-th listed replica is wl_p[k], and the start of cell g is
// p0 + E[g] - wl_p[k].  The starts of the other replicas' cells stay as they were, and the first
// cell of every replica starts at its p0, so cell_start[c + 1] ends every cell c.  Three kernels on
// a fixed grid of SCAN_BLOCKS blocks: each block's share of the sequence is summed, the block sums
// are scanned, and each block scans its share again from its offset and writes the starts.
constexpr int SCAN_BLOCKS = 256;
constexpr int SCAN_T = 1024;

__device__ __forceinline__ void scan_share(const DevState& s, int& lo, int& hi) {
  const int tot = s.wl_c[*s.wl_n];
  const int seg = ((tot + SCAN_BLOCKS - 1) / SCAN_BLOCKS + SCAN_T - 1) / SCAN_T * SCAN_T;
  lo = min(tot, (int)blockIdx.x * seg);
  hi = min(tot, lo + seg);
}

// block sum of v (all threads); the total in every thread
__device__ __forceinline__ int block_sum_int(int v, int* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  int t = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
  return t;
}

__global__ void __launch_bounds__(SCAN_T) k_wscan_sum(DevState s) {
  __shared__ int red[SCAN_T / 32];
  int lo, hi;
  scan_share(s, lo, hi);
  const int n = *s.wl_n;
  int v = 0;
  for (int g = lo + threadIdx.x; g < hi; g += SCAN_T) {
    int r, c;
    wl_map_warp(s.wl_c, s.wl_rep, n, g, r, c);
    v += s.cell_count[s.reps[r].cell_off + c];
  }
  v = block_sum_int(v, red);
  if (threadIdx.x == 0) s.scan_blk[blockIdx.x] = v;
}

// exclusive scan of the SCAN_BLOCKS block sums (one block)
__global__ void __launch_bounds__(SCAN_T) k_wscan_blocks(DevState s) {
  __shared__ int warp_tot[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int v = threadIdx.x < SCAN_BLOCKS ? s.scan_blk[threadIdx.x] : 0;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    const int t = warp_tot[lane];
    int u = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, u, o);
      if (lane >= o) u += y;
    }
    warp_tot[lane] = u - t;
  }
  __syncthreads();
  if (threadIdx.x < SCAN_BLOCKS) s.scan_blk[SCAN_BLOCKS + threadIdx.x] = x - v + warp_tot[wid];
}

__global__ void __launch_bounds__(SCAN_T) k_wscan_write(DevState s) {
  __shared__ int warp_tot[32];
  __shared__ int carry;
  int lo, hi;
  scan_share(s, lo, hi);
  const int n = *s.wl_n;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = s.scan_blk[SCAN_BLOCKS + blockIdx.x];
  __syncthreads();
  for (int base = lo; base < hi; base += SCAN_T) {
    const int g = base + threadIdx.x;
    int r = 0, c = 0, k = 0, v = 0;
    if (g < hi) {
      k = wl_map_warp(s.wl_c, s.wl_rep, n, g, r, c);
      v = s.cell_count[s.reps[r].cell_off + c];
    }
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
      const int t = warp_tot[lane];
      int u = t;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, u, o);
        if (lane >= o) u += y;
      }
      warp_tot[lane] = u - t;
    }
    __syncthreads();
    const int e = carry + warp_tot[wid] + x - v;  // E[g]
    if (g < hi) s.cell_start[s.reps[r].cell_off + c] = s.reps[r].p0 + e - s.wl_p[k];
    __syncthreads();
    if (threadIdx.x == SCAN_T - 1) carry = e + v;
    __syncthreads();
  }
}

__global__ void k_place(DevState s) {
  WL_FOR(wl_p, g) {
    int r, loc;
    wl_map_warp(s.wl_p, s.wl_rep, wl_cnt_, g, r, loc);
    const int i = s.reps[r].p0 + loc;
    s.perm[s.cell_start[s.cell_of[i]] + s.rank[i]] = i;
  }
}

// compare-exchange of (tag, slot) pairs by tag
__device__ __forceinline__ void cmpx(int (&t)[8], int (&p)[8], int i, int j) {
  if (t[j] < t[i]) {
    const int u = t[i], q = p[i];
    t[i] = t[j]; p[i] = p[j];
    t[j] = u; p[j] = q;
  }
}

__global__ void k_sort_cells(DevState s) {
  WL_FOR(wl_c, g) {
  int r, lc;
  wl_map_warp(s.wl_c, s.wl_rep, wl_cnt_, g, r, lc);
  const int c = s.reps[r].cell_off + lc;
  int b = s.cell_start[c], n = s.cell_count[c];
  s.cell_count[c] = 0;  // the last reader of the count: zero again for the next rebuild's k_bin
  if (n <= 1) continue;
  if (n <= 8) {
    // a cell of up to 8: all its slots and tags loaded at once (two dependent loads, not a chain
    // per element), sorted in registers by a fixed network (Batcher's odd-even merge for 8, its
    // 4-input form for up to 4) with the unused places padded by the largest tag
    int p[8], t[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) p[k] = k < n ? s.perm[b + k] : 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) t[k] = k < n ? s.tag[p[k]] : 0x7fffffff;
    cmpx(t, p, 0, 1); cmpx(t, p, 2, 3); cmpx(t, p, 0, 2); cmpx(t, p, 1, 3); cmpx(t, p, 1, 2);
    if (n > 4) {
      cmpx(t, p, 4, 5); cmpx(t, p, 6, 7); cmpx(t, p, 4, 6); cmpx(t, p, 5, 7); cmpx(t, p, 5, 6);
      // merge of the two sorted halves
      cmpx(t, p, 0, 4); cmpx(t, p, 1, 5); cmpx(t, p, 2, 6); cmpx(t, p, 3, 7);
      cmpx(t, p, 2, 4); cmpx(t, p, 3, 5);
      cmpx(t, p, 1, 2); cmpx(t, p, 3, 4); cmpx(t, p, 5, 6);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (k < n) s.perm[b + k] = p[k];
    continue;
  }
  for (int k = 1; k < n; ++k) {  // insertion sort by tag
    int p = s.perm[b + k];
    int t = s.tag[p];
    int m = k - 1;
    while (m >= 0 && s.tag[s.perm[b + m]] > t) {
      s.perm[b + m + 1] = s.perm[b + m];
      --m;
    }
    s.perm[b + m + 1] = p;
  }
  }
}

__global__ void k_permute(DevState s) {
  WL_FOR(wl_p, g) {
  int r, loc;
  wl_map_warp(s.wl_p, s.wl_rep, wl_cnt_, g, r, loc);
  const int i = s.reps[r].p0 + loc;
  int o = s.perm[i];
  s.tmp[0][i] = s.rx[o];
  s.tmp[1][i] = s.ry[o];
  s.tmp[2][i] = s.rz[o];
  s.tmp[3][i] = s.vx[o];
  s.tmp[4][i] = s.vy[o];
  s.tmp[5][i] = s.vz[o];
  const int wo = s.info[o];
  if (s.permute_accel || !info_mobile(wo)) {
    s.tmp[6][i] = s.ax[o];
    s.tmp[7][i] = s.ay[o];
    s.tmp[8][i] = s.az[o];
  }
  s.tmp_tag[i] = s.tag[o];
  s.tmp_info[i] = wo;
  }
}

// Writes the pair-kernel views of slot i and returns the fixed-point position (w in q.w).
__device__ __forceinline__ int4 write_views(const DevState& s, int i, const RepDesc& R, double x, double y, double z,
                                            double vx, double vy, double vz, int w, int t) {
  int4 q;
  q.x = to_fx_periodic(x, R.sfx[0]);
  q.y = to_fx_periodic(y, R.sfx[1]);
  q.z = to_fx_z(z, R.sfx[2]);
  q.w = w;
  if (s.mixed) {
    s.pfx[i] = q;
    s.vf[i] = make_float4(d2f_fast(vx), d2f_fast(vy), d2f_fast(vz), __int_as_float(t));
  } else {
    s.pd[i] = mk_dbl4(x, y, z, __longlong_as_double((long long)w));
    s.vd[i] = mk_dbl4(vx, vy, vz, __longlong_as_double((long long)t));
  }
  return q;
}

__global__ void k_copyback(DevState s) {
  WL_FOR(wl_p, g) {
  int rr, loc;
  wl_map_warp(s.wl_p, s.wl_rep, wl_cnt_, g, rr, loc);
  const int i = s.reps[rr].p0 + loc;
  double x = s.tmp[0][i], y = s.tmp[1][i], z = s.tmp[2][i];
  double vx = s.tmp[3][i], vy = s.tmp[4][i], vz = s.tmp[5][i];
  s.rx[i] = x; s.ry[i] = y; s.rz[i] = z;
  s.vx[i] = vx; s.vy[i] = vy; s.vz[i] = vz;
  int t = s.tmp_tag[i], w = s.tmp_info[i];
  if (s.permute_accel || !info_mobile(w)) {
    s.ax[i] = s.tmp[6][i]; s.ay[i] = s.tmp[7][i]; s.az[i] = s.tmp[8][i];
  }
  s.tag[i] = t;
  s.info[i] = w;
  s.slot_of_tag[t] = i;
  const RepDesc& R = s.reps[info_rep(w)];
  int4 q = write_views(s, i, R, x, y, z, vx, vy, vz, w, t);
  q.w = 0;
  s.ref[i] = q;
  }
}

// Full Verlet list: every mobile particle lists all j (mobile or wall) with r^2 < (rc_ij+skin)^2.
// One thread per particle.  Cells are at least 1/H of the list cut-off wide (H = 2 by default),
// and the (2H+1)^3 cells around a particle are walked as (2H+1)^2 x-rows: the cells of a row are
// consecutive in the sorted order unless the row wraps in x, so a row is one contiguous slot range
// (two when it wraps).
// Rows whose y/z distance from the particle exceeds the largest list cut-off of its type are
// skipped, and each kept row is trimmed in x to the cells within that cut-off, which removes
// about half of the candidates.  Each thread stages its first NL_STAGE entries in shared memory
// (row stride NL_STAGE|1 keeps the banks distinct) and the block writes them out row by row: the
// k-th neighbours of 128 consecutive particles are 128 consecutive ints of nbr, so every store is
// coalesced (scattered 4-byte stores into the column-major list cost read-modify-writes in HBM).
// The fixed staging size keeps the shared memory (17 KB per block) independent of the list
// capacity, so eight blocks fit on an SM.  The blocks take chunks of the replicas being rebuilt
// from a queue.
// entries per particle staged in shared memory (the first NL_STAGE rows of the list are written
// coalesced; a particle with more neighbours writes the rest straight to the list)
constexpr int NL_STAGE = 32;

template <bool MIXED, bool UNI, int H, int HX = H>
__global__ void __launch_bounds__(NL_BLOCK, 8) k_nlist(DevState s) {
  const int nwl = *s.wl_n;
  const int nchunks = s.wl_k[nwl];
  if ((int)blockIdx.x >= nchunks) return;
  __shared__ int nl_sh[NL_BLOCK * (NL_STAGE | 1)];
  __shared__ float rl2f[NPAIR];
  __shared__ double rl2d[NPAIR];
  __shared__ float rlmax[MAXT];
  __shared__ int blk_max;
  __shared__ int chunk;
  const int cap = s.nbr_cap;
  int* mine = nl_sh + threadIdx.x * (NL_STAGE | 1);
  for (int k = threadIdx.x; k < NPAIR; k += blockDim.x) {
    rl2d[k] = s.tabd[k].rlist2;
    rl2f[k] = s.tabf ? s.tabf[k].rlist2 : 0.f;
  }
  if (threadIdx.x < MAXT) {  // largest list cut-off of each type, with the culling margin
    double m = 0.;
    for (int t = 0; t < MAXT; ++t) m = fmax(m, s.tabd[threadIdx.x * MAXT + t].rlist2);
    rlmax[threadIdx.x] = (float)m * 1.0004f;
  }
  for (;;) {
  // the next chunk from the queue (chunks differ in cost: a queue keeps the blocks busy)
  __syncthreads();
  if (threadIdx.x == 0) chunk = atomicAdd(s.wl_n + 1, 1);
  __syncthreads();
  const int ch = chunk;
  if (ch >= nchunks) break;
  int rc, kc;  // the chunk's replica and its index there (the same for the whole block)
  wl_map(s.wl_k, s.wl_rep, nwl, ch, rc, kc);
  const int i0 = s.reps[rc].p0 + kc * NL_BLOCK, i1 = min(s.reps[rc].p0 + s.reps[rc].n_part, i0 + NL_BLOCK);
  const int i = i0 + threadIdx.x;
  const bool doit = i < i1;
  const int w = doit ? s.info[i] : 0;
  if (threadIdx.x == 0) blk_max = 0;
  __syncthreads();
  int cnt = 0, found = 0;  // entries stored, neighbours found (more when the list overflows)
  if (doit && info_mobile(w)) {
    const RepDesc& R = s.reps[info_rep(w)];
    const int ti = info_type(w);
    int ix, iy, iz;
    int4 qi = make_int4(0, 0, 0, 0);
    double x = 0., y = 0., z = 0.;
    if (MIXED) {
      qi = s.pfx[i];
      ix = (int)(((unsigned long long)(unsigned)qi.x * (unsigned)R.nc[0]) >> 32);
      iy = (int)(((unsigned long long)(unsigned)qi.y * (unsigned)R.nc[1]) >> 32);
      iz = (int)(((long long)qi.z * R.nc[2]) >> 30);
      iz = min(max(iz, 0), R.nc[2] - 1);
    } else {
      x = s.rx[i]; y = s.ry[i]; z = s.rz[i];
      cell_coords(R, x, y, z, ix, iy, iz);
    }
    // coarse conversion (512 fixed-point units); rl2f carries a 2e-4 margin
    const float ux = R.ufx_f[0] * 512.f, uy = R.ufx_f[1] * 512.f, uz = R.ufx_f[2] * 512.f;
    const int nx = R.nc[0];
    // Row culling and x trimming: a cell is skipped when its distance from the particle, taken
    // from the cell edges, is beyond the largest list cut-off of the particle's type times 1.0004
    // (the candidate test below has a 1.0002 margin; the coarse position is off by < 1e-5 sigma).
    // (no FP64 and no conversion instructions here: both run on the slow FP64 pipe)
    float px, py, pz;  // position in cell units
    if (MIXED) {
      px = (__int_as_float(0x4B000000 | ((unsigned)qi.x >> 9)) - 8388608.0f) * R.cpu_f[0];
      py = (__int_as_float(0x4B000000 | ((unsigned)qi.y >> 9)) - 8388608.0f) * R.cpu_f[1];
      pz = i2f_coarse(qi.z, 9) * R.cpu_f[2];
    } else {
      px = (float)(x * R.inv_lc[0]);
      py = (float)(y * R.inv_lc[1]);
      pz = (float)(z * R.inv_lc[2]);
    }
    const float lx = R.lc_f[0], ly = R.lc_f[1], lz = R.lc_f[2];
    const float rl2max = rlmax[ti];
    const float rl_uni = s.rl2_uni;  // UNI: one list cut-off for every pair (2e-4 margin included)
    auto fl = [](int v) { return i2f_coarse(v, 0); };  // exact for small integers
    auto gap2 = [](float d, float l) {  // squared gap of d cell widths (0 when the particle is past the edge)
      d = fmaxf(d, 0.f) * l;
      return d * d;
    };
    float gxp[HX], gxm[HX];  // squared gaps to the cells ix + k and ix - k, k = 1..HX
#pragma unroll
    for (int k = 1; k <= HX; ++k) {
      gxp[k - 1] = gap2(fl(ix + k) - px, lx);
      gxm[k - 1] = gap2(px - fl(ix - k + 1), lx);
    }
    for (int dz = -H; dz <= H; ++dz) {
      const int cz = iz + dz;
      if (cz < 0 || cz >= R.nc[2]) continue;
      const float rz2 = rl2max - ((dz > 0) ? gap2(fl(cz) - pz, lz) : (dz < 0 ? gap2(pz - fl(cz + 1), lz) : 0.f));
      for (int dy = -H; dy <= H; ++dy) {
        int cy = iy + dy;
        const float rem2 = rz2 - ((dy > 0) ? gap2(fl(cy) - py, ly) : (dy < 0 ? gap2(py - fl(cy + 1), ly) : 0.f));
        if (rem2 <= 0.f) continue;  // the whole row is beyond the list cut-off
        int xa = ix, xb = ix;
#pragma unroll
        for (int k = 0; k < HX; ++k) {
          xa -= gxm[k] < rem2;
          xb += gxp[k] < rem2;
        }
        cy += (cy < 0) ? R.nc[1] : 0;
        cy -= (cy >= R.nc[1]) ? R.nc[1] : 0;
        const int row = R.cell_off + (cz * R.nc[1] + cy) * nx;
        // x-runs of cells xa..xb: one contiguous slot range, or two when the row wraps; the
        // scan has one entry past the last cell, so cell_start[c + 1] ends cell c
        int xa0, xb0, xa1 = 0, xb1 = -1;
        if (xa < 0) { xa0 = 0; xb0 = xb; xa1 = nx + xa; xb1 = nx - 1; }
        else if (xb >= nx) { xa0 = xa; xb0 = nx - 1; xa1 = 0; xb1 = xb - nx; }
        else { xa0 = xa; xb0 = xb; }
        const int nseg = (xb1 >= xa1) ? 2 : 1;
        int sb[2], se[2];
        sb[0] = s.cell_start[row + xa0];
        se[0] = s.cell_start[row + xb0 + 1];
        if (nseg == 2) {
          sb[1] = s.cell_start[row + xa1];
          se[1] = s.cell_start[row + xb1 + 1];
        }
        for (int g = 0; g < nseg; ++g) {
          // not unrolled: the rows are short (a few candidates in 3x3x3 cells), and unrolling by
          // 2 / 4 / 8 measured 0.6 / 2.9 / 3.8 % slower on a rebuild of 256 brush replicas
#pragma unroll 1
          for (int j = sb[g]; j < se[g]; ++j) {
            int wj;
            bool hit;
            if (MIXED) {
              const int4 qj = s.pfx[j];
              wj = qj.w;
              const float ddx = i2f_coarse(fx_diff(qi.x, qj.x), 9) * ux;
              const float ddy = i2f_coarse(fx_diff(qi.y, qj.y), 9) * uy;
              const float ddz = i2f_coarse(fx_diff(qi.z, qj.z), 9) * uz;
              hit = ddx * ddx + ddy * ddy + ddz * ddz < (UNI ? rl_uni : rl2f[ti * MAXT + info_type(wj)]);
            } else {
              wj = s.info[j];
              const double ddx = mic_ref(x - s.rx[j], R.L[0], R.invL[0]);
              const double ddy = mic_ref(y - s.ry[j], R.L[1], R.invL[1]);
              const double ddz = z - s.rz[j];
              hit = ddx * ddx + ddy * ddy + ddz * ddz < rl2d[ti * MAXT + info_type(wj)];
            }
            if (hit && j != i) {
              if (cnt < NL_STAGE) mine[cnt] = j;
              else if (cnt < cap) s.nbr[(size_t)cnt * s.Np + i] = j;  // rare: past the staged rows
              ++cnt;
            }
          }
        }
      }
    }
    found = cnt;
    if (cnt > cap) {
      atomicOr(s.status, ST_NLIST_OVERFLOW);
      cnt = cap;
    }
  }
  atomicMax(&blk_max, found);  // the true count, so that the host grows the capacity past it
  __syncthreads();
  if (threadIdx.x == 0) atomicMax(s.status + 1, (unsigned)blk_max);  // largest count, for the host
  const int mx = min(blk_max, NL_STAGE);
  if (doit) {
    for (int k = 0; k < mx; ++k)
      if (k < cnt) s.nbr[(size_t)k * s.Np + i] = mine[k];
    s.nn[i] = cnt;
  }
  __syncthreads();  // the staging area and blk_max are reused by the next chunk
  }
}


// End of a rebuild: counts it (when some replica was flagged) and the flagged replicas' rebuilds,
// then clears the flags.
__global__ void k_clear_flags(int* flag, int nrep, long long* rebuilds, long long* rep_rebuilds) {
  const bool any = flag[0] != 0;
  __syncthreads();
  for (int r = threadIdx.x; r < nrep; r += blockDim.x) {
    if (flag[1 + r]) {
      rep_rebuilds[r] += 1;
      flag[1 + r] = 0;
    }
  }
  if (threadIdx.x == 0 && any) {
    *rebuilds += 1;
    flag[0] = 0;
  }
}

void launch_rebuild(const DevState& s, cudaStream_t st, bool force) {
  const int B = 256;
  // fixed grids that stride over the work list: a few waves of the GPU, at most what the largest
  // work (every particle or cell) fills
  const int gN = std::min((s.N + B - 1) / B, s.nsm * 8);
  const int gC = std::min((s.ncell_tot + B - 1) / B, s.nsm * 8);
  k_worklist<<<1, WL_THREADS, 0, st>>>(s, force);
  k_bin<<<gN, B, 0, st>>>(s);
  k_wscan_sum<<<SCAN_BLOCKS, SCAN_T, 0, st>>>(s);
  k_wscan_blocks<<<1, SCAN_T, 0, st>>>(s);
  k_wscan_write<<<SCAN_BLOCKS, SCAN_T, 0, st>>>(s);
  k_place<<<gN, B, 0, st>>>(s);
  k_sort_cells<<<gC, B, 0, st>>>(s);
  k_permute<<<gN, B, 0, st>>>(s);
  k_copyback<<<gN, B, 0, st>>>(s);
  const int var = s.mixed ? (s.rl2_uni > 0.f ? 2 : 1) : 0;
  using KernT = void (*)(DevState);
  const KernT kerns[3][3] = {{k_nlist<false, false, 1>, k_nlist<true, false, 1>, k_nlist<true, true, 1>},
                             {k_nlist<false, false, 2>, k_nlist<true, false, 2>, k_nlist<true, true, 2>},
                             {k_nlist<false, false, 3>, k_nlist<true, false, 3>, k_nlist<true, true, 3>}};
  // cells finer along x alone (with 3x3 rows in y, z)
  const KernT kx[2][3] = {{k_nlist<false, false, 1, 2>, k_nlist<true, false, 1, 2>, k_nlist<true, true, 1, 2>},
                          {k_nlist<false, false, 1, 3>, k_nlist<true, false, 1, 3>, k_nlist<true, true, 1, 3>}};
  const KernT kern = (s.nl_hx != s.nl_h) ? kx[s.nl_hx - 2][var] : kerns[s.nl_h - 1][var];
  const int gl = std::min((s.N + NL_BLOCK - 1) / NL_BLOCK, s.nsm * 8);
  kern<<<gl, NL_BLOCK, 0, st>>>(s);
  k_clear_flags<<<1, 256, 0, st>>>(s.rebuild_flag, s.nrep, s.rebuilds, s.rep_rebuilds);
}

// ---------------------------------------------------------------------------------------------
// Parity exports with the reference's own grid (cell_list.f90:129-213, 285-433)
// ---------------------------------------------------------------------------------------------
__global__ void k_ref_cells(DevState s, int rep, double il0, double il1, double il2, int n0, int n1, int n2,
                            int* __restrict__ cell_of_tag, int* __restrict__ counts) {
  const RepDesc& R = s.reps[rep];
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= R.n_mon_tot) return;
  int i = s.slot_of_tag[R.p0 + t];
  double r[3] = {s.rx[i], s.ry[i], s.rz[i]};
  double il[3] = {il0, il1, il2};
  int nc[3] = {n0, n1, n2};
  int pc = 1, pf = 1;
  for (int d = 0; d < 3; ++d) {
    int c = (int)(r[d] * il[d]);
    c = min(max(c, 0), nc[d] - 1);
    pc += pf * c;
    pf *= nc[d];
  }
  cell_of_tag[t] = pc;
  atomicAdd(&counts[pc], 1);
}

void launch_ref_cells(const DevState& s, cudaStream_t st, int rep, const double* il, const int* nc, int* cell_of_tag,
                      int* counts) {
  int n = s.N;  // upper bound; the kernel checks the replica's own count
  k_ref_cells<<<(n + 255) / 256, 256, 0, st>>>(s, rep, il[0], il[1], il[2], nc[0], nc[1], nc[2], cell_of_tag, counts);
}

__global__ void k_cell_neigh(int n0, int n1, int n2, int n_nei, int* __restrict__ out) {
  int in_cell = blockIdx.x * blockDim.x + threadIdx.x + 1;
  int nct = n0 * n1 * n2;
  if (in_cell > nct) return;
  int z_cell = (in_cell - 1) / (n0 * n1) + 1;
  int y_cell = (in_cell - n0 * n1 * (z_cell - 1) - 1) / n0 + 1;
  int x_cell = in_cell - n0 * n1 * (z_cell - 1) - n0 * (y_cell - 1);
  int* o = out + (size_t)(in_cell - 1) * n_nei;
  int il = 0;
  int lo = (n_nei == 13) ? 1 : 0, hi = (n_nei == 13) ? 3 : 4, ilo = 2, ihi = (n_nei == 13) ? 3 : 4;
  for (int i = ilo; i <= ihi; ++i)
    for (int j = lo; j <= hi; ++j) {
      if (i == 2 && j <= 1) continue;
      for (int k = lo; k <= hi; ++k) {
        if (i == 2 && j == 2 && k >= 3) continue;
        int jc = in_cell + i - 2 + (j - 2) * n0 + (k - 2) * n1 * n0;
        if (jc == in_cell) continue;
        if (n_nei == 13) {
          if (x_cell == 1 && i == 1) jc += n0;
          if (x_cell == n0 && i == 3) jc -= n0;
          if (y_cell == 1 && j == 1) jc += n0 * n1;
          if (y_cell == n1 && j == 3) jc -= n0 * n1;
        } else {
          if (x_cell + i - 2 > n0) jc -= n0;
          if (y_cell + j - 2 < 1) jc += n0 * n1;
          if (y_cell + j - 2 > n1) jc -= n0 * n1;
        }
        if (z_cell + k - 2 < 1) jc = 0;
        if (z_cell + k - 2 > n2) jc = 0;
        o[il++] = jc;
      }
    }
}

void launch_cell_neigh(const int* nc, int n_nei, int* out, cudaStream_t st) {
  int nct = nc[0] * nc[1] * nc[2];
  k_cell_neigh<<<(nct + 127) / 128, 128, 0, st>>>(nc[0], nc[1], nc[2], n_nei, out);
}

}  // namespace mfa
