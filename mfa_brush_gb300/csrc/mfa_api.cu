// mfa_api.cu -- the C ABI of include/mfa_gpu.h: contexts, per-routine drop-ins, the fused
// graph-captured step, host<->device movement, parity exports and timing.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/mfa_gpu.h"
#include "mfa_obs.cuh"
#include "mfa_state.cuh"

using namespace mfa;

struct mfa_ctx {
  int device = 0;
  cudaStream_t st = nullptr;
  cudaStream_t st2 = nullptr;  // captures the bodies of conditional graph nodes
  cudaStream_t stc = nullptr;  // host <-> device copies of mfa_set_state / mfa_sync_to_host
  cudaEvent_t ev_io[5] = {};   // their ordering against the compute stream
  mfa_params P;
  mfa_options opt;
  std::vector<mfa_system> sys;
  int nrep = 0, N = 0, Np = 0;
  SimConst C;
  DevState S;
  std::vector<RepDesc> hreps;
  RepDesc* dreps = nullptr;
  PairEntry<float>* dtabf = nullptr;
  PairEntry<double>* dtabd = nullptr;
  double* acc_step = nullptr;  // [NOBS][nrep]
  double* acc_call = nullptr;
  double* rec = nullptr;       // [NOBS][nrep] last record of mfa_step
  double* prof = nullptr;
  long long n_obs = 0;
  std::vector<double> v_coul_self, v_ww;
  std::vector<double> v_ff_walls;  // LJ energy of the fixed wall beads among themselves (WALL 1)
  std::vector<KSpace> Ks;  // k-space of each replica (its own box, k-set and charged particles)
  bool kspace = false;
  bool fuse_integ = false;  // mfa_step runs the integration of its plain steps in the pair kernel
  unsigned* h_status = nullptr;  // pinned: [0] status bits, [1] largest list count seen
  cudaEvent_t ev_status = nullptr;  // recorded after each copy of the status words into h_status
  bool grow_pending = false;     // the list capacity is to be raised before the next step
  bool overflow_reported = false;  // the current list overflow was returned to the caller already
  long long* h_rebuilds = nullptr;
  long long last_rebuilds = 0;
  long long host_steps = 0;      // steps completed (host view)
  int last_source = 0;           // 0 none, 1 mfa_step record, 2 per-routine accumulators
  std::map<std::tuple<int, int, int, int>, std::pair<cudaGraphExec_t, long long>> graphs;
  cudaEvent_t ev[16];
  long long launches = 0;
  std::vector<void*> allocs;
  double* stage = nullptr;  // 4 x 3N doubles for host <-> device state movement, made on first use
  double* obs = nullptr;    // [nrep][9] of mfa_observe and of the averages
  double* avg = nullptr;    // [nrep][NAVG] observation averages (options.observe)
  double* series = nullptr; // [series_capacity][O_VIR][nrep] energy records (options.series_capacity)
  long long* series_step = nullptr;  // [series_capacity] steps done at each record
  long long* series_head = nullptr;  // [1] records written
  long long series_read = 0;         // records returned to the caller
  // device addresses of the file-scope scratch of mfa_pair_list_static, looked up at the first
  // call of that entry point on this context (with the context's device current)
  int* static_pairs = nullptr;
  unsigned long long* static_count = nullptr;
  std::string err;
  double rl_max = 0.;
};

namespace {

const char* kFamNames[MFA_NKFAM] = {"rebuild", "pair", "bonded", "integrate", "kspace", "profiles", "record",
                                    "positions", "rebuild_all"};

int fail(mfa_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

#define CK(call)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      return fail(ctx, MFA_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));         \
  } while (0)

#define RET(x)              \
  do {                      \
    int r__ = (x);          \
    if (r__) return r__;    \
  } while (0)

template <typename T>
int dalloc(mfa_ctx* ctx, T** p, size_t n) {
  void* q = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc(&q, n * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();  // an allocation failure is not sticky: later launch checks must not see it
    return fail(ctx, MFA_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  ctx->allocs.push_back(q);
  *p = (T*)q;
  return MFA_OK;
}

#define DA(p, n)                                   \
  do {                                             \
    int r_ = dalloc(ctx, &(p), (size_t)(n));       \
    if (r_ != MFA_OK) return r_;                   \
  } while (0)

Acc acc_of(double* a, int nrep) { return Acc{a, nrep}; }

// The list capacity is raised before the next step when the largest list count of the rebuilds
// so far has passed 85 % of it (or the lists overflowed), so that a density fluctuation later in
// the run does not overflow them.
void note_list_count(mfa_ctx* ctx) {
  if (ctx->h_status[1] * 20u > (unsigned)ctx->S.nbr_cap * 17u && ctx->S.nbr_cap < NL_CAP_MAX)
    ctx->grow_pending = true;
}

int check_status(mfa_ctx* ctx) {
  CK(cudaStreamSynchronize(ctx->st));
  unsigned s = ctx->h_status[0];
  note_list_count(ctx);
  if (s & ST_NAN) return fail(ctx, MFA_ERR_NAN, "non-finite position detected");
  if (s & ST_OUT_OF_BOX) return fail(ctx, MFA_ERR_OUT_OF_BOX, "a particle left the channel");
  if (s & ST_NLIST_OVERFLOW) {
    ctx->overflow_reported = true;
    return fail(ctx, MFA_ERR_NLIST_OVERFLOW, "neighbour list capacity exceeded");
  }
  return MFA_OK;
}

int post_status(mfa_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->h_status, ctx->S.status, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaEventRecord(ctx->ev_status, ctx->st));
  return MFA_OK;
}

// Non-blocking look at the status words of the last post_status: when that copy has arrived (no
// copy into h_status is then in flight), a list count past 85 % of the capacity schedules the
// growth, and an overflow of an earlier rebuild is reported.  When it has not arrived yet, the
// next call looks again.  Lets a caller that only ever calls mfa_step get the growth too.
int poll_status(mfa_ctx* ctx) {
  const cudaError_t q = cudaEventQuery(ctx->ev_status);
  if (q == cudaErrorNotReady) return MFA_OK;
  CK(q);
  note_list_count(ctx);
  if (ctx->h_status[0] & ST_NLIST_OVERFLOW) return MFA_ERR_NLIST_OVERFLOW;
  return MFA_OK;
}

__global__ void k_clear_overflow(unsigned* status) {
  atomicAnd(status, ~ST_NLIST_OVERFLOW);
  status[1] = 0u;
}

// rebuild of the flagged replicas (all of them when forced); counts and clears the flags
constexpr int kRebuildLaunches = 11;
void rebuild(mfa_ctx* ctx, bool force) {
  launch_rebuild(ctx->S, ctx->st, force);
  ctx->launches += kRebuildLaunches;
}

// Graph form of the skin check: the IF body (the eleven rebuild kernels) runs only on steps whose
// position update raised the flag of some replica; other steps launch nothing.
__global__ void k_cond_rebuild(const int* flag, cudaGraphConditionalHandle h) {
  cudaGraphSetConditional(h, flag[0] ? 1u : 0u);
}

int capture_conditional_rebuild(mfa_ctx* ctx, const DevState& S) {
  cudaStream_t st = ctx->st;
  cudaStreamCaptureStatus cs;
  cudaGraph_t graph;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &graph, &deps, nullptr, &nd));
  cudaGraphConditionalHandle h;
  CK(cudaGraphConditionalHandleCreate(&h, graph, 0, 0));
  k_cond_rebuild<<<1, 1, 0, st>>>(S.rebuild_flag, h);
  CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &graph, &deps, nullptr, &nd));
  cudaGraphNodeParams cp = {};  // aggregate initialisation: all reserved fields zero
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeIf;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, graph, deps, nullptr, nd, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  CK(cudaStreamBeginCaptureToGraph(ctx->st2, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  launch_rebuild(S, ctx->st2, false);  // the flagged replicas (the flags stay set until its last kernel)
  cudaGraph_t captured;
  CK(cudaStreamEndCapture(ctx->st2, &captured));
  CK(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  return MFA_OK;
}

int bonded_mask(const mfa_ctx* ctx) {
  int m = 1;
  if (ctx->P.flags.bending) m |= 2;
  if (ctx->P.flags.bending_melt) m |= 4;
  if (ctx->P.flags.orientation) m |= 8;
  return m;
}

bool any_chains(const mfa_ctx* ctx) {
  for (auto& s : ctx->sys)
    if ((s.n_mon > 1 && s.n_chain > 0) || (s.n_mon_d > 1 && s.n_chain_d > 0) || (s.n_mon_e > 1 && s.n_chain_e > 0))
      return true;
  return false;
}

void fill_energies(const mfa_ctx* ctx, const double* acc, int rep, mfa_energies* e) {
  record_energies(acc, ctx->nrep, rep, ctx->hreps[rep], ctx->C, e);
  e->step = ctx->sys[rep].s_time + ctx->host_steps;
}

void fill_virial(const mfa_ctx* ctx, const double* acc, int rep, mfa_virial* o) {
  record_virial(acc, ctx->nrep, rep, ctx->hreps[rep], ctx->C, o);
  o->step = ctx->sys[rep].s_time + ctx->host_steps;
}

// ewald_k(0) (ewald_k.f90:37-124): the k-vectors in the reference's enumeration order, G(k),
// and the list of charged particles, of replica rep (the particles p0 .. p0 + n_mon_tot - 1 of the
// batch; a_type holds the whole batch).
int setup_kspace(mfa_ctx* ctx, const int32_t* a_type, int rep) {
  const mfa_system& s = ctx->sys[rep];
  const int p0 = ctx->hreps[rep].p0;
  const mfa_params& p = ctx->P;
  const double pi = (double)3.1415926536f;  // mfa_common.f90:315
  const double* L = s.boundary;
  const double z_slab = 2.;
  const double dk[3] = {2. * pi * (1. / L[0]), 2. * pi * (1. / L[1]), 2. * pi / (L[2] + z_slab * L[2])};
  const double k_c = (dk[0] + dk[1]) * (double)p.n_kmax / 2.;
  const int nx = (int)(k_c / dk[0]), ny = (int)(k_c / dk[1]), nz = (int)(k_c / dk[2]);
  const double fac_alpha = 1. / (4. * p.alpha_c);
  std::vector<int4> kn;
  std::vector<double> kv, kf;
  for (int kz = 0; kz <= nz; ++kz)
    for (int ky = -ny; ky <= ny; ++ky)
      for (int kx = -nx; kx <= nx; ++kx) {
        const double a1 = (double)kx * dk[0], b1 = (double)ky * dk[1], c1 = (double)kz * dk[2];
        const double rk2 = a1 * a1 + b1 * b1 + c1 * c1;
        if (rk2 > k_c * k_c) continue;
        if (kz == 0 && ky == 0 && kx == 0) continue;
        if (kz == 0 && kx + ky < 0) continue;
        if (kz == 0 && -kx == ky && ky > 0) continue;
        kn.push_back(make_int4(kx, ky, kz, 0));
        const double k0 = dk[0] * kx, k1 = dk[1] * ky, k2 = dk[2] * kz;
        kv.push_back(k0);
        kv.push_back(k1);
        kv.push_back(k2);
        const double kk = k0 * k0 + k1 * k1 + k2 * k2;
        kf.push_back((1. / kk) * std::exp(-kk * fac_alpha));
      }
  KSpace& K = ctx->Ks[rep];
  std::memset(&K, 0, sizeof K);
  K.nk = (int)kn.size();
  K.nxm = nx;
  K.nym = ny;
  K.nzm = nz;
  K.ncol = (nx + 1) + (ny + 1) + (nz + 1);
  K.cx = dk[0] / (2. * M_PI);
  K.cy = dk[1] / (2. * M_PI);
  K.cz = dk[2] / (2. * M_PI);
  K.inv_V = (1. / L[0]) * (1. / L[1]) / (L[2] * (1. + z_slab));
  K.lz_half = L[2] / 2.;
  K.rep = rep;
  K.plain = ctx->opt.kspace_plain_sums ? 1 : 0;
  std::vector<int> qt;
  std::vector<double> qv;
  for (int t = 0; t < s.n_mon_tot; ++t)
    if (p.charge[a_type[p0 + t] - 1] != 0.) {
      qt.push_back(p0 + t);  // the batch's tag
      qv.push_back(p.charge[a_type[p0 + t] - 1]);
    }
  K.nq = (int)qt.size();
  std::vector<float> qvf(qv.begin(), qv.end());
  // rows: maximal runs of k with one (ky, kz)
  std::vector<int4> rows;
  std::vector<int> krow(K.nk);
  for (int k = 0; k < K.nk; ++k) {
    if (k == 0 || kn[k].y != kn[k - 1].y || kn[k].z != kn[k - 1].z) rows.push_back(make_int4(k, k, kn[k].y, kn[k].z));
    rows.back().y = k + 1;
    krow[k] = (int)rows.size() - 1;
  }
  K.nrows = (int)rows.size();
  // slots of a row: nx = -nxm .. -nxm + 4 qx - 1 (the dense slot table of the force kernel)
  K.qx = (2 * nx + 1 + 3) / 4;
  // force chunks of whole rows: KS_FR for the dense kernel; for the one-k-at-a-time kernel as
  // many as let its shared-memory tables fit (the X table alone grows with nxm)
  const bool dense = kspace_dense(K, ctx->S.mixed);
  std::vector<int> chunk_row;
  for (int frows = KS_FR;; frows /= 2) {
    chunk_row.clear();
    for (int r = 0; r < K.nrows; r += frows) chunk_row.push_back(r);
    chunk_row.push_back(K.nrows);
    K.nkchunks = (int)chunk_row.size() - 1;
    K.fchunk_k_max = K.fchunk_rows_max = 1;
    for (int c = 0; c < K.nkchunks; ++c) {
      K.fchunk_k_max = std::max(K.fchunk_k_max, rows[chunk_row[c + 1] - 1].y - rows[chunk_row[c]].x);
      K.fchunk_rows_max = std::max(K.fchunk_rows_max, chunk_row[c + 1] - chunk_row[c]);
    }
    if (dense || kspace_force_smem(K, ctx->S.mixed) <= KS_SMEM_MAX) break;
    if (frows == 1)
      return fail(ctx, MFA_ERR_CAPACITY, "ewald_k: the k-set is too wide in x for the force kernel's tables");
  }
  // force order of the rows (dense kernel): by slot range, widest first, so that the KS_FR rows
  // of a chunk share a narrow window of slots
  std::vector<int> frow(K.nrows), fpos(K.nrows);
  for (int r = 0; r < K.nrows; ++r) frow[r] = r;
  auto lo_of = [&](int r) { return kn[rows[r].x].x + nx; };
  auto hi_of = [&](int r) { return lo_of(r) + rows[r].y - rows[r].x - 1; };
  std::stable_sort(frow.begin(), frow.end(), [&](int a, int b) {
    const int wa = hi_of(a) - lo_of(a), wb = hi_of(b) - lo_of(b);
    return wa != wb ? wa > wb : lo_of(a) < lo_of(b);
  });
  for (int f = 0; f < K.nrows; ++f) fpos[frow[f]] = f;
  std::vector<int2> fwin(K.nkchunks);
  for (int c = 0; c < K.nkchunks; ++c) {
    int lo = 1 << 30, hi = -1;
    for (int f = c * KS_FR; f < std::min(K.nrows, (c + 1) * KS_FR); ++f) {
      lo = std::min(lo, lo_of(frow[f]));
      hi = std::max(hi, hi_of(frow[f]));
    }
    fwin[c] = make_int2(lo, hi);
  }
  // rho particle chunks: one wave of three blocks per SM, chunks a multiple of the 32-particle tile
  const int kb = (K.nrows + 63) / 64 * ((2 * nx + 1 + 31) / 32);  // k_ks_rho: 64 rows x 32 slots
  int pch = std::max(1, std::min(256, (3 * 152 + kb - 1) / kb));
  K.pchunk = std::max(32, ((K.nq + pch - 1) / pch + 31) / 32 * 32);
  K.npchunks = std::max(1, (K.nq + K.pchunk - 1) / K.pchunk);
  DA(K.kn, K.nk);
  DA(K.kvec, 3 * K.nk);
  DA(K.kfac, K.nk);
  DA(K.mz, 1);
  DA(K.rows, K.nrows);
  DA(K.krow, K.nk);
  DA(K.chunk_row, K.nkchunks + 1);
  DA(K.frow, K.nrows);
  DA(K.fpos, K.nrows);
  DA(K.fwin, K.nkchunks);
  DA(K.rho_part, (size_t)K.npchunks * 2 * K.nk);
  DA(K.fpart, (size_t)K.nkchunks * std::max(K.nq, 1) * 3);
  DA(K.red_part, 8 * KS_RED_MAX);
  DA(K.ticket, 2);
  DA(K.qtag, K.nq);
  DA(K.qval, K.nq);
  DA(K.qvalf, K.nq);
  if (ctx->S.mixed) {
    DA(K.tabf, (size_t)K.nq * K.ncol);
    DA(K.kdf, K.nk);
    DA(K.wdense, (size_t)K.nrows * 4 * K.qx);
  } else {
    DA(K.tabd, (size_t)K.nq * K.ncol);
    DA(K.kdd, K.nk);
  }
  cudaStream_t st = ctx->st;
  CK(cudaMemcpyAsync(K.kn, kn.data(), sizeof(int4) * K.nk, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(K.kvec, kv.data(), sizeof(double) * 3 * K.nk, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(K.kfac, kf.data(), sizeof(double) * K.nk, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(K.rows, rows.data(), sizeof(int4) * K.nrows, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(K.krow, krow.data(), sizeof(int) * K.nk, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(K.chunk_row, chunk_row.data(), sizeof(int) * (K.nkchunks + 1), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(K.frow, frow.data(), sizeof(int) * K.nrows, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(K.fpos, fpos.data(), sizeof(int) * K.nrows, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(K.fwin, fwin.data(), sizeof(int2) * K.nkchunks, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(K.ticket, 0, 2 * sizeof(unsigned), st));
  if (K.wdense) CK(cudaMemsetAsync(K.wdense, 0, sizeof(float4) * K.nrows * 4 * K.qx, st));
  if (K.nq) {
    CK(cudaMemcpyAsync(K.qtag, qt.data(), sizeof(int) * K.nq, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(K.qval, qv.data(), sizeof(double) * K.nq, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(K.qvalf, qvf.data(), sizeof(float) * K.nq, cudaMemcpyHostToDevice, st));
  }
  CK(cudaStreamSynchronize(st));
  CK((cudaError_t)kspace_prepare(K, ctx->S.mixed));
  ctx->kspace = true;
  return MFA_OK;
}

}  // namespace

extern "C" {

const char* mfa_version(void) { return "mfa_gb300 1.0 (sm_103a)"; }

int mfa_device_count(int32_t* n) {
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  if (e != cudaSuccess) c = 0;
  if (n) *n = c;
  return MFA_OK;
}

void mfa_default_options(mfa_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof *o);
  o->precision = MFA_PREC_MIXED;
  o->device = 0;
  o->skin = 0.3;
  o->nbr_capacity = 0;
  o->energy_every = 10;
  o->use_graphs = 1;
  o->block_size = 0;
  o->profile_from_step = 0;
}

int mfa_init(const mfa_params* p, const mfa_system* sys, const int32_t* a_type, const double* r0, const double* v,
             const double* a, const mfa_options* opt, mfa_ctx** out) {
  return mfa_batch_init(p, 1, sys, a_type, r0, v, a, opt, out);
}

int mfa_batch_init(const mfa_params* p, int32_t n_rep, const mfa_system* sysv, const int32_t* a_type,
                   const double* r0, const double* v, const double* a, const mfa_options* opt, mfa_ctx** out) {
  if (!out) return MFA_ERR_ARG;
  *out = nullptr;
  if (!p || n_rep < 1 || !sysv || !a_type || !r0) return MFA_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MFA_ERR_NO_DEVICE;
  mfa_ctx* ctx = new mfa_ctx();
  *out = ctx;
  ctx->P = *p;
  if (opt) ctx->opt = *opt; else mfa_default_options(&ctx->opt);
  if (ctx->opt.energy_every < 1) ctx->opt.energy_every = 10;
  if (ctx->opt.skin <= 0) ctx->opt.skin = 0.3;
  ctx->device = ctx->opt.device;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&ctx->st2, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&ctx->stc, cudaStreamNonBlocking));
  for (int k = 0; k < 16; ++k) CK(cudaEventCreate(&ctx->ev[k]));
  for (int k = 0; k < 5; ++k) CK(cudaEventCreateWithFlags(&ctx->ev_io[k], cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&ctx->ev_status, cudaEventDisableTiming));
  const mfa_flags& F = p->flags;
  if (p->n_type < 1 || p->n_type > MFA_MAX_TYPES) return fail(ctx, MFA_ERR_ARG, "n_type out of range");
  if (F.symmetry != 0) return fail(ctx, MFA_ERR_UNSUPPORTED, "only SYMMETRY 0 (channel) is built");
  if (p->compat & MFA_COMPAT_EWALD_I_ONLY)
    return fail(ctx, MFA_ERR_UNSUPPORTED, "Coulomb force on i only depends on the reference's loop order");
  const bool charged = F.system == 2 || F.system == 3;
  ctx->nrep = n_rep;
  ctx->sys.assign(sysv, sysv + n_rep);
  long long N = 0;
  for (auto& s : ctx->sys) {
    if (s.n_part < s.n_mon_tot || s.n_mon_tot < 0) return fail(ctx, MFA_ERR_ARG, "n_part < n_mon_tot");
    N += s.n_part;
  }
  if (N < 1 || N > (1ll << 30)) return fail(ctx, MFA_ERR_ARG, "particle count out of range");
  ctx->N = (int)N;
  ctx->Np = (int)((N + 31) / 32 * 32);
  // ---- scalars --------------------------------------------------------------------------------
  SimConst& C = ctx->C;
  std::memset(&C, 0, sizeof C);
  C.n_type = p->n_type;
  C.thermostat_dpd = F.thermostat == 0;
  C.dpd_weight1 = F.dpd_weight == 1;
  C.force_switch_on = F.force_switch_on;
  C.poiseuille = F.poiseuille;
  C.bending = F.bending;
  C.bending_melt = F.bending_melt;
  C.orientation = F.orientation;
  C.bend_form = p->bend_form;
  C.charged = charged;
  C.wall = F.wall;
  C.dt = p->dt;
  C.va_wall[0] = p->va_wall[0];
  C.va_wall[1] = p->va_wall[1];
  C.move_walls = F.wall == 1 && (p->va_wall[0] != 0. || p->va_wall[1] != 0.);
  C.half_dt = 0.5 * p->dt;
  C.half_dt2 = 0.5 * (p->dt * p->dt);
  for (int t = 0; t < MAXT; ++t) {
    C.mass[t] = p->mass_type[t];
    C.inv_mass[t] = p->mass_type[t] != 0. ? 1. / p->mass_type[t] : 0.;
    C.sigma_wall[t] = p->sigma_wall[t];
    C.a_wall[t] = p->a_wall[t];
    C.charge[t] = p->charge[t];
  }
  C.gamma = p->friction1;
  C.sig = p->sig;
  C.r2min_init = p->r_2_min_init;
  C.r2min_time = p->r_2_min_time;
  C.a_w = p->a_w;
  C.k_chain = p->k_chain;
  C.inv_r_chain_2 = p->inv_r_chain_2;
  C.fene_xmax = (double)0.98f;
  C.k_bend = p->k_bend;
  C.alpha_eq = p->alpha_eq;
  C.k_or = p->k_or;
  C.alpha_or = p->alpha_or;
  C.bend_small = (double)0.000001f;
  for (int d = 0; d < 3; ++d) C.const_force[d] = p->const_force[d];
  C.sqrt_alpha = p->sqrt_alpha;
  C.alpha_c = p->alpha_c;
  C.inv_sqrt_pi = p->inv_sqrt_pi;
  C.coul_rc2 = p->rc_coul_2;
  const double skin = ctx->opt.skin;
  C.skin_half2 = 0.25 * skin * skin;
  C.hist_dim = p->hist_dim > 0 ? p->hist_dim : 200;
  C.dt_f = (float)C.dt;
  C.skin_half2_f = (float)C.skin_half2;
  C.a_w_f = (float)C.a_w;
  for (int t = 0; t < MAXT; ++t) {
    C.mass_f[t] = (float)C.mass[t];
    C.inv_mass_f[t] = (float)C.inv_mass[t];
    C.sigma_wall_f[t] = (float)C.sigma_wall[t];
    C.a_wall_f[t] = (float)C.a_wall[t];
  }
  for (int d = 0; d < 3; ++d) C.cforce_f[d] = (float)C.const_force[d];
  C.sig_f = (float)C.sig; C.gamma_f = (float)C.gamma; C.coul_rc2_f = (float)C.coul_rc2;
  C.sqrt_alpha_f = (float)C.sqrt_alpha; C.inv_sqrt_pi_f = (float)C.inv_sqrt_pi; C.alpha_c_f = (float)C.alpha_c;
  C.k_chain_f = (float)C.k_chain; C.inv_r_chain_2_f = (float)C.inv_r_chain_2; C.fene_xmax_f = (float)C.fene_xmax;
  C.k_bend_f = (float)C.k_bend; C.alpha_eq_f = (float)C.alpha_eq; C.k_or_f = (float)C.k_or;
  C.alpha_or_f = (float)C.alpha_or; C.bend_small_f = (float)C.bend_small;
  if (C.hist_dim > MFA_HIST_DIM_MAX) return fail(ctx, MFA_ERR_CAPACITY, "hist_dim exceeds MFA_HIST_DIM_MAX");
  // ---- pair tables ----------------------------------------------------------------------------
  std::vector<PairEntry<float>> tf(NPAIR);
  std::vector<PairEntry<double>> td(NPAIR);
  const int W = p->n_type - 1;
  double rl_max = 0.;
  for (int i = 0; i < MAXT; ++i)
    for (int j = 0; j < MAXT; ++j) {
      PairEntry<double> e;
      std::memset(&e, 0, sizeof e);
      const int k = i * MAXT + j;
      if (i < p->n_type && j < p->n_type) {
        e.range2 = p->range_2[k];
        e.eps4 = p->epsil[k];
        e.sig2 = p->sigma_2[k];
        e.shift = p->e_shift[k];
        e.inv_rc = std::sqrt(p->inv_range_2[k]);
        const bool wallpair = F.wall == 1 && (i == W || j == W);
        int fl = 0;
        if (e.range2 > 0.) fl |= PF_LJ;
        double rc = std::sqrt(e.range2);
        if (F.thermostat == 0) {
          if (p->r_cut_dpd_2 == 0.) {
            if (e.range2 > 0. && !wallpair) fl |= PF_DPD_LJ;
          } else if (i != 0 && j != 0 && !wallpair) {
            fl |= PF_DPD_OWN;
            e.dpd_rc2 = p->r_cut_dpd_2;
            e.inv_dpd_rc = 1. / std::sqrt(p->r_cut_dpd_2);
            rc = std::max(rc, std::sqrt(p->r_cut_dpd_2));
          }
        }
        if (charged && p->charge[i] * p->charge[j] != 0.) {
          fl |= PF_COUL;
          e.qq = p->charge[i] * p->charge[j];
          if (p->rc_coul_2 > 0.) rc = std::max(rc, std::sqrt(p->rc_coul_2));
        }
        e.flags = fl;
        e.rlist2 = rc > 0. ? (rc + skin) * (rc + skin) : 0.;
        e.screen2 = rc * rc;
        if (rc > 0.) rl_max = std::max(rl_max, rc + skin);
      }
      td[k] = e;
      PairEntry<float>& g = tf[k];
      g.range2 = (float)e.range2; g.eps4 = (float)e.eps4; g.sig2 = (float)e.sig2; g.shift = (float)e.shift;
      g.inv_rc = (float)e.inv_rc; g.rlist2 = (float)e.rlist2; g.dpd_rc2 = (float)e.dpd_rc2;
      g.inv_dpd_rc = (float)e.inv_dpd_rc; g.qq = (float)e.qq; g.flags = e.flags;
      g.screen2 = (float)(e.screen2 * 1.0002);
      g.rlist2 = (float)(e.rlist2 * 1.0002);
    }
  if (rl_max <= 0.) rl_max = 1.0 + skin;
  ctx->rl_max = rl_max;
  {  // uniform cut-offs: every nonzero list cut-off of the present types equal (and the screens)
    double lo = 1e300, hi = 0., slo = 1e300, shi = 0.;
    for (int i = 0; i < p->n_type; ++i)
      for (int j = 0; j < p->n_type; ++j) {
        const PairEntry<double>& e = td[i * MAXT + j];
        if (e.rlist2 > 0.) { lo = std::min(lo, e.rlist2); hi = std::max(hi, e.rlist2); }
        if (e.screen2 > 0.) { slo = std::min(slo, e.screen2); shi = std::max(shi, e.screen2); }
      }
    const bool uni = hi > 0. && hi == lo && shi == slo;
    C.rl2_uni_f = uni ? (float)(hi * 1.0002) : 0.f;
    C.scr2_uni_f = uni ? (float)(shi * 1.0002) : 0.f;
  }
  // ---- replicas -------------------------------------------------------------------------------
  ctx->hreps.resize(n_rep);
  ctx->v_coul_self.assign(n_rep, 0.);
  ctx->v_ww.assign(n_rep, 0.);
  ctx->v_ff_walls.assign(n_rep, 0.);
  int cell_off = 0, p0 = 0;
  double dens_max = 0.;
  // list-build cells per list cut-off: as asked, else the fewest (the largest cells: fewest rows
  // to walk) that every replica's box holds 2h+1 of in x and y
  int nl_h = ctx->opt.list_cells;
  if (nl_h < 0 || nl_h > 3) return fail(ctx, MFA_ERR_ARG, "list_cells must be 0, 1, 2 or 3");
  if (nl_h == 0) {
    nl_h = 1;
    for (int r = 0; r < n_rep; ++r)
      for (int d = 0; d < 2; ++d)
        while (nl_h < 3 && std::floor(ctx->sys[r].boundary[d] / (rl_max / nl_h)) < 2 * nl_h + 1) ++nl_h;
  }
  // along x: as asked, else 2 with 3x3 rows in y, z when every box holds 5 such cells in x (the
  // x-runs then follow the cut-off sphere more closely), else as in y, z
  int nl_hx = ctx->opt.list_cells_x;
  if (nl_hx == 0) {
    nl_hx = nl_h;
    bool fits = nl_h == 1;
    for (int r = 0; r < n_rep; ++r) fits = fits && std::floor(ctx->sys[r].boundary[0] / (rl_max / 2)) >= 5;
    if (fits) nl_hx = 2;
  }
  if (nl_hx < 1 || nl_hx > 3 || (nl_hx != nl_h && nl_h != 1))
    return fail(ctx, MFA_ERR_ARG, "list_cells_x must be 0, or 1, 2 or 3 with list_cells 1");
  for (int r = 0; r < n_rep; ++r) {
    const mfa_system& s = ctx->sys[r];
    RepDesc& R = ctx->hreps[r];
    std::memset(&R, 0, sizeof R);
    for (int d = 0; d < 3; ++d) {
      if (!(s.boundary[d] > 0.)) return fail(ctx, MFA_ERR_ARG, "box length must be positive");
      R.L[d] = s.boundary[d];
      R.invL[d] = 1. / s.boundary[d];
      R.sfx[d] = (d < 2) ? 4294967296.0 / s.boundary[d] : 1073741824.0 / s.boundary[d];
      R.ufx[d] = 1. / R.sfx[d];
      R.ufx_f[d] = (float)R.ufx[d];
      // list cells of at least 1/h of the list cut-off: the (2h+1)^3 stencil covers every
      // neighbour, and 2h+1 cells in x and y keep each cell of a stencil row distinct
      const int h = (d == 0) ? nl_hx : nl_h;
      int nc = (int)std::floor(s.boundary[d] / (rl_max / h));
      if (nc < 1) nc = 1;
      if (d < 2 && nc < 2 * h + 1)
        return fail(ctx, MFA_ERR_UNSUPPORTED,
                    "box shorter than (2 + 1/list_cells)*(r_cut_max+skin) in x or y");
      R.nc[d] = nc;
      R.inv_lc[d] = (double)nc / s.boundary[d];
      R.lc_f[d] = (float)(s.boundary[d] / nc);
      R.cpu_f[d] = (float)(512. * nc / ((d < 2) ? 4294967296.0 : 1073741824.0));
      if (d == 2) {
        R.zlim_f[0] = (float)(-s.boundary[2] / nc);
        R.zlim_f[1] = (float)(s.boundary[2] + s.boundary[2] / nc);
      }
    }
    R.ncell = R.nc[0] * R.nc[1] * R.nc[2];
    R.cell_off = cell_off;
    cell_off += R.ncell;
    R.p0 = p0;
    R.n_part = s.n_part;
    R.n_mon_tot = s.n_mon_tot;
    R.n_mon = s.n_mon; R.n_chain = s.n_chain; R.n_mon_d = s.n_mon_d; R.n_chain_d = s.n_chain_d;
    R.n_mon_e = s.n_mon_e; R.n_chain_e = s.n_chain_e;
    R.part_init_d = s.n_mon * s.n_chain;
    R.part_init_e = R.part_init_d + s.n_mon_d * s.n_chain_d;
    if (R.part_init_e + s.n_mon_e * s.n_chain_e != s.n_mon_tot)
      return fail(ctx, MFA_ERR_ARG, "n_mon_tot differs from the chain counts");
    R.seed = s.seed;
    R.s_time = s.s_time;
    R.lz_half = s.boundary[2] / 2.;
    const double D = s.boundary[2];
    if (F.wall == 2)  // wall_wall.f90:45-48
      ctx->v_ww[r] = 2.0 * (std::fabs(p->a_w) * std::pow(p->sigma_w / D, 9) - p->a_w * std::pow(p->sigma_w / D, 3));
    R.v_ww = ctx->v_ww[r];
    R.v_ffw = 0.;  // set below for explicit walls
    R.v_cself = 0.;
    R.inv_n = (F.system == 2) ? 1. / (double)s.n_mon_tot : 1. / (double)(s.n_mon_tot - s.n_chain);
    R.hist_inv_dz = 1. / (D / (double)C.hist_dim);
    std::memcpy(&R.Lbits[0], &R.L[0], 8);
    std::memcpy(&R.Lbits[1], &R.L[1], 8);
    p0 += s.n_part;
    dens_max = std::max(dens_max, (double)s.n_part / (s.boundary[0] * s.boundary[1] * D));
    if (F.wall == 1) {
      // Explicit walls: the reference's Verlet list holds every particle, wall beads included
      // (binning.f90:25,56), so v_fluid_fluid also sums the wall-wall pairs (fluid_fluid.f90:61).
      // The wall beads never move: that part is a constant, summed here once.
      double vw = 0.;
      for (int i = s.n_mon_tot; i < s.n_part; ++i)
        for (int j = i + 1; j < s.n_part; ++j) {
          const double* ri = r0 + 3 * (size_t)(R.p0 + i);
          const double* rj = r0 + 3 * (size_t)(R.p0 + j);
          double d[3] = {ri[0] - rj[0], ri[1] - rj[1], ri[2] - rj[2]};
          for (int c = 0; c < 2; ++c) d[c] -= s.boundary[c] * std::nearbyint(d[c] / s.boundary[c]);
          const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
          const PairEntry<double>& e = td[(a_type[R.p0 + i] - 1) * MAXT + (a_type[R.p0 + j] - 1)];
          if (r2 < e.range2) {
            const double s2 = e.sig2 / r2, s6 = s2 * s2 * s2;
            vw += e.eps4 * ((s6 * s6 - s6) - e.shift);
          }
        }
      ctx->v_ff_walls[r] = vw;
      R.v_ffw = vw;
    }
    if (charged) {
      double vs = 0.;
      for (int t = 0; t < s.n_mon_tot; ++t) vs -= p->charge[a_type[R.p0 + t] - 1] * p->charge[a_type[R.p0 + t] - 1];
      ctx->v_coul_self[r] = vs * p->sqrt_alpha / std::sqrt((double)3.1415926536f);
      R.v_cself = ctx->v_coul_self[r];
    }
  }
  // ---- per-particle info ----------------------------------------------------------------------
  std::vector<int> info(ctx->N), iota(ctx->N);
  for (int r = 0; r < n_rep; ++r) {
    const RepDesc& R = ctx->hreps[r];
    for (int t = 0; t < R.n_part; ++t) {
      int g = R.p0 + t;
      int ty = a_type[g] - 1;
      if (ty < 0 || ty >= p->n_type) return fail(ctx, MFA_ERR_ARG, "particle type out of range");
      int mob = t < R.n_mon_tot;
      int head = (t < R.part_init_d && R.n_mon > 0 && t % R.n_mon == 0) ? 1 : 0;
      int sp = (t < R.part_init_d) ? 0 : (t < R.part_init_e ? 1 : (t < R.n_mon_tot ? 2 : 3));
      info[g] = ty | (mob << 4) | (head << 5) | (sp << 6) | (r << 8);
      iota[g] = g;
    }
  }
  // ---- device memory --------------------------------------------------------------------------
  DevState& S = ctx->S;
  std::memset(&S, 0, sizeof S);
  S.N = ctx->N;
  S.Np = ctx->Np;
  S.nrep = n_rep;
  S.mixed = ctx->opt.precision == MFA_PREC_MIXED;
  const size_t Nn = ctx->Np;
  double** dst[12] = {&S.rx, &S.ry, &S.rz, &S.vx, &S.vy, &S.vz, &S.ax, &S.ay, &S.az, &S.fx, &S.fy, &S.fz};
  for (auto d : dst) DA(*d, Nn);
  for (int k = 0; k < 9; ++k) DA(S.tmp[k], Nn);
  DA(S.tag, Nn); DA(S.info, Nn); DA(S.tmp_tag, Nn); DA(S.tmp_info, Nn); DA(S.slot_of_tag, Nn);
  if (S.mixed) {
    DA(S.pfx, Nn); DA(S.vf, Nn); DA(S.f4, Nn);
    DA(S.pfx_alt, Nn); DA(S.vf_alt, Nn);
  } else {
    DA(S.pd, Nn); DA(S.vd, Nn);
  }
  DA(S.ref, Nn);
  DA(S.nn, Nn);
  DA(S.cell_of, Nn); DA(S.rank, Nn); DA(S.perm, Nn);
  S.ncell_tot = cell_off;
  DA(S.cell_count, cell_off + 1);  // zero between rebuilds: k_bin counts up, k_sort_cells zeroes
  DA(S.cell_start, cell_off + 1);
  DA(S.scan_blk, 2 * 256);  // the cell-start scan's block sums and offsets
  DA(S.rebuild_flag, 1 + n_rep);
  DA(S.steps_alt, 1);
  S.sync_alt = 0;
  S.permute_accel = 1;
  DA(S.pair_q, 2);
  DA(S.wl_rep, n_rep + 1);
  DA(S.wl_p, n_rep + 1);
  DA(S.wl_c, n_rep + 1);
  DA(S.wl_k, n_rep + 1);
  DA(S.wl_n, 2);
  CK(cudaDeviceGetAttribute(&S.nsm, cudaDevAttrMultiProcessorCount, ctx->device));
  DA(S.cell_rep, cell_off);
  DA(S.rebuilds, 1);
  DA(S.rep_rebuilds, n_rep);
  DA(S.status, 2);  // [0] status bits, [1] largest list count of the rebuilds so far
  DA(S.steps_done, 1);
  DA(ctx->dreps, n_rep);
  DA(ctx->dtabf, NPAIR);
  DA(ctx->dtabd, NPAIR);
  DA(ctx->acc_step, NOBS * n_rep);
  DA(ctx->acc_call, NOBS * n_rep);
  DA(ctx->rec, NOBS * n_rep);
  DA(ctx->prof, (size_t)n_rep * C.hist_dim * 21);
  DA(ctx->obs, (size_t)9 * n_rep);
  if (ctx->opt.observe) DA(ctx->avg, (size_t)NAVG * n_rep);
  if (ctx->opt.series_capacity < 0) return fail(ctx, MFA_ERR_ARG, "series_capacity < 0");
  if (ctx->opt.series_capacity > 0) {
    DA(ctx->series, (size_t)ctx->opt.series_capacity * O_VIR * n_rep);
    DA(ctx->series_step, ctx->opt.series_capacity);
  }
  DA(ctx->series_head, 1);
  CK(cudaMallocHost(&ctx->h_status, 2 * sizeof(unsigned)));
  CK(cudaMallocHost(&ctx->h_rebuilds, sizeof(long long)));
  ctx->h_status[0] = ctx->h_status[1] = 0;
  S.reps = ctx->dreps;
  S.tabf = ctx->dtabf;
  S.tabd = ctx->dtabd;
  S.rl2_uni = S.mixed ? C.rl2_uni_f : 0.f;
  S.nl_h = nl_h;
  S.nl_hx = nl_hx;
  if (ctx->opt.pair_schedule < 0 || ctx->opt.pair_schedule > 1)
    return fail(ctx, MFA_ERR_ARG, "pair_schedule must be 0 or 1");
  S.pair_persist = ctx->opt.pair_schedule;
  // neighbour capacity: 2x the mean count of the densest replica + 32, at least 48
  int cap = ctx->opt.nbr_capacity;
  if (cap <= 0) {
    double est = 4. / 3. * M_PI * rl_max * rl_max * rl_max * dens_max;
    cap = (int)std::ceil(2.0 * est) + 32;
    cap = std::max(cap, 48);
  }
  cap = std::min(cap, NL_CAP_MAX);
  S.nbr_cap = cap;
  DA(S.nbr, (size_t)cap * Nn);
  cudaStream_t st = ctx->st;
  CK(cudaMemcpyAsync(ctx->dreps, ctx->hreps.data(), sizeof(RepDesc) * n_rep, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->dtabf, tf.data(), sizeof(PairEntry<float>) * NPAIR, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(ctx->dtabd, td.data(), sizeof(PairEntry<double>) * NPAIR, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(S.info, info.data(), sizeof(int) * ctx->N, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(S.tag, iota.data(), sizeof(int) * ctx->N, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(S.slot_of_tag, iota.data(), sizeof(int) * ctx->N, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(S.rebuild_flag, 0, sizeof(int) * (1 + n_rep), st));
  CK(cudaMemsetAsync(S.cell_count, 0, sizeof(int) * (cell_off + 1), st));
  CK(cudaMemsetAsync(S.pair_q, 0, sizeof(int) * 2, st));
  {
    std::vector<int> cr(std::max(cell_off, 1));
    for (int r = 0; r < n_rep; ++r)
      for (int c = 0; c < ctx->hreps[r].ncell; ++c) cr[ctx->hreps[r].cell_off + c] = r;
    CK(cudaMemcpy(S.cell_rep, cr.data(), sizeof(int) * cell_off, cudaMemcpyHostToDevice));
  }
  CK(cudaMemsetAsync(S.rep_rebuilds, 0, sizeof(long long) * n_rep, st));
  CK(cudaMemsetAsync(S.status, 0, 2 * sizeof(unsigned), st));
  CK(cudaMemsetAsync(S.steps_done, 0, sizeof(long long), st));
  CK(cudaMemsetAsync(S.steps_alt, 0, sizeof(long long), st));
  CK(cudaMemsetAsync(S.rebuilds, 0, sizeof(long long), st));
  CK(cudaMemsetAsync(ctx->acc_step, 0, sizeof(double) * NOBS * n_rep, st));
  CK(cudaMemsetAsync(ctx->acc_call, 0, sizeof(double) * NOBS * n_rep, st));
  CK(cudaMemsetAsync(ctx->rec, 0, sizeof(double) * NOBS * n_rep, st));
  CK(cudaMemsetAsync(ctx->prof, 0, sizeof(double) * n_rep * C.hist_dim * 21, st));
  if (ctx->avg) CK(cudaMemsetAsync(ctx->avg, 0, sizeof(double) * NAVG * n_rep, st));
  CK(cudaMemsetAsync(ctx->series_head, 0, sizeof(long long), st));
  for (int k = 9; k < 12; ++k) CK(cudaMemsetAsync(*dst[k], 0, sizeof(double) * Nn, st));
  // ---- state upload (canonical AoS -> slots) --------------------------------------------------
  {
    double *dr = nullptr, *dv = nullptr, *dac = nullptr;
    size_t n3 = 3 * (size_t)ctx->N;
    CK(cudaMalloc(&dr, n3 * 8));
    CK(cudaMalloc(&dv, n3 * 8));
    CK(cudaMalloc(&dac, n3 * 8));
    CK(cudaMemcpyAsync(dr, r0, n3 * 8, cudaMemcpyHostToDevice, st));
    if (v) CK(cudaMemcpyAsync(dv, v, n3 * 8, cudaMemcpyHostToDevice, st)); else CK(cudaMemsetAsync(dv, 0, n3 * 8, st));
    if (a) CK(cudaMemcpyAsync(dac, a, n3 * 8, cudaMemcpyHostToDevice, st)); else CK(cudaMemsetAsync(dac, 0, n3 * 8, st));
    launch_scatter_state(S, st, dr, dv, dac);
    launch_init_views(S, st);
    CK(cudaStreamSynchronize(st));
    cudaFree(dr);
    cudaFree(dv);
    cudaFree(dac);
  }
  // ---- k-space --------------------------------------------------------------------------------
  if (charged && p->n_kmax > 0) {
    ctx->Ks.assign(n_rep, KSpace{});
    for (int rep = 0; rep < n_rep; ++rep) {
      int r = setup_kspace(ctx, a_type, rep);
      if (r != MFA_OK) return r;
    }
  }
  if (ctx->opt.separate_integrator < 0 || ctx->opt.separate_integrator > 1)
    return fail(ctx, MFA_ERR_ARG, "separate_integrator must be 0 or 1");
  // the integration fused into the pair kernel: mixed precision, no k-space (its forces come after
  // the pair kernel's), one block per tile
  ctx->fuse_integ = S.mixed && !ctx->kspace && !ctx->opt.separate_integrator && !S.pair_persist;
  // ---- initial sort + list, then size the list from the observed maximum ------------------------
  rebuild(ctx, true);
  RET(post_status(ctx));
  int rc = check_status(ctx);
  if (rc == MFA_ERR_NLIST_OVERFLOW || rc == MFA_OK) {
    std::vector<int> nn(ctx->N);
    CK(cudaMemcpy(nn.data(), S.nn, sizeof(int) * ctx->N, cudaMemcpyDeviceToHost));
    int mx = 0;
    for (int x : nn) mx = std::max(mx, x);
    if (rc == MFA_ERR_NLIST_OVERFLOW || (ctx->opt.nbr_capacity <= 0 && mx * 3 / 2 + 16 > cap)) {
      // grow and redo: count beyond the capacity is not stored, so retry with a larger one
      int newcap = std::max(cap * 2, mx * 3 / 2 + 32);
      if (rc == MFA_ERR_NLIST_OVERFLOW) newcap = std::max(newcap, cap * 3);
      auto it = std::find(ctx->allocs.begin(), ctx->allocs.end(), (void*)S.nbr);
      if (it != ctx->allocs.end()) { cudaFree(*it); ctx->allocs.erase(it); }
      newcap = std::min(newcap, NL_CAP_MAX);
      if (newcap <= cap) return fail(ctx, MFA_ERR_CAPACITY, "more neighbours per particle than the list builder holds");
      S.nbr_cap = newcap;
      DA(S.nbr, (size_t)newcap * Nn);
      CK(cudaMemsetAsync(S.status, 0, 2 * sizeof(unsigned), st));
      ctx->h_status[0] = ctx->h_status[1] = 0;
      rebuild(ctx, true);
      RET(post_status(ctx));
      rc = check_status(ctx);
    }
  }
  if (rc != MFA_OK) return rc;
  CK(cudaMemcpy(ctx->h_rebuilds, ctx->S.rebuilds, sizeof(long long), cudaMemcpyDeviceToHost));
  ctx->last_rebuilds = *ctx->h_rebuilds;
  return MFA_OK;
}

int mfa_destroy(mfa_ctx* ctx) {
  if (!ctx) return MFA_OK;
  if (ctx->st) cudaStreamSynchronize(ctx->st);
  for (auto& g : ctx->graphs) cudaGraphExecDestroy(g.second.first);
  for (void* p : ctx->allocs) cudaFree(p);
  if (ctx->h_status) cudaFreeHost(ctx->h_status);
  if (ctx->h_rebuilds) cudaFreeHost(ctx->h_rebuilds);
  for (int k = 0; k < 16; ++k)
    if (ctx->ev[k]) cudaEventDestroy(ctx->ev[k]);
  if (ctx->st) cudaStreamDestroy(ctx->st);
  for (int k = 0; k < 5; ++k)
    if (ctx->ev_io[k]) cudaEventDestroy(ctx->ev_io[k]);
  if (ctx->ev_status) cudaEventDestroy(ctx->ev_status);
  if (ctx->st2) cudaStreamDestroy(ctx->st2);
  if (ctx->stc) cudaStreamDestroy(ctx->stc);
  delete ctx;
  return MFA_OK;
}

const char* mfa_last_error(const mfa_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int mfa_synchronize(mfa_ctx* ctx) {
  if (!ctx) return MFA_ERR_ARG;
  RET(post_status(ctx));
  return check_status(ctx);
}

void* mfa_stream(mfa_ctx* ctx) { return ctx ? (void*)ctx->st : nullptr; }

int mfa_n_particles(const mfa_ctx* ctx, int64_t* n_total, int32_t* n_rep) {
  if (!ctx) return MFA_ERR_ARG;
  if (n_total) *n_total = ctx->N;
  if (n_rep) *n_rep = ctx->nrep;
  return MFA_OK;
}

// ---- per-routine drop-ins -------------------------------------------------------------------
// A drop-in clears the accumulator slots it fills; from then on the energy, virial and head-force
// readers take the per-routine accumulators (until the next mfa_step record).
static int zero_call_slot(mfa_ctx* ctx, int slot, int n = 1) {
  CK(cudaMemsetAsync(ctx->acc_call + (size_t)slot * ctx->nrep, 0, sizeof(double) * ctx->nrep * n, ctx->st));
  ctx->last_source = 2;
  return MFA_OK;
}
// the 9 virial slots of a group (each drop-in replaces its own group)
static int zero_call_group(mfa_ctx* ctx, int group) { return zero_call_slot(ctx, O_VIR + 9 * group, 9); }

static int read_call_slot(mfa_ctx* ctx, int slot, double* out, double add_self) {
  if (!out) return MFA_OK;
  CK(cudaMemcpyAsync(out, ctx->acc_call + (size_t)slot * ctx->nrep, sizeof(double) * ctx->nrep,
                     cudaMemcpyDeviceToHost, ctx->st));
  RET(post_status(ctx));
  int r = check_status(ctx);
  if (r != MFA_OK) return r;
  if (add_self != 0.)
    for (int k = 0; k < ctx->nrep; ++k) out[k] += ctx->v_coul_self[k];
  return MFA_OK;
}

static int grow_lists(mfa_ctx* ctx);

static int prepare_step(mfa_ctx* ctx);

int mfa_verlet_positions(mfa_ctx* ctx) {
  if (!ctx) return MFA_ERR_ARG;
  RET(prepare_step(ctx));
  launch_integrate(ctx->S, ctx->C, ctx->st, 0, false, false, acc_of(ctx->acc_call, ctx->nrep));
  ctx->launches += 1;
  rebuild(ctx, false);
  CK(cudaGetLastError());
  return MFA_OK;
}

int mfa_check_skin(mfa_ctx* ctx, int32_t* rebuilt) {
  if (!ctx) return MFA_ERR_ARG;
  rebuild(ctx, false);
  CK(cudaMemcpyAsync(ctx->h_rebuilds, ctx->S.rebuilds, sizeof(long long), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  if (rebuilt) *rebuilt = (*ctx->h_rebuilds != ctx->last_rebuilds) ? 1 : 0;
  ctx->last_rebuilds = *ctx->h_rebuilds;
  return MFA_OK;
}

int mfa_zero_force(mfa_ctx* ctx) {
  if (!ctx) return MFA_ERR_ARG;
  CK(cudaMemsetAsync(ctx->S.fx, 0, sizeof(double) * ctx->N, ctx->st));
  CK(cudaMemsetAsync(ctx->S.fy, 0, sizeof(double) * ctx->N, ctx->st));
  CK(cudaMemsetAsync(ctx->S.fz, 0, sizeof(double) * ctx->N, ctx->st));
  return MFA_OK;
}

int mfa_fluid_fluid(mfa_ctx* ctx, double* v_ff, double* v_coul) {
  if (!ctx) return MFA_ERR_ARG;
  int r;
  if ((r = zero_call_slot(ctx, O_VFF)) || (r = zero_call_slot(ctx, O_VCOUL)) || (r = zero_call_group(ctx, V_PAIR)))
    return r;
  launch_pair(ctx->S, ctx->C, ctx->st, true, true, acc_of(ctx->acc_call, ctx->nrep), ctx->opt.block_size);
  ctx->launches += 1;
  CK(cudaGetLastError());
  ctx->last_source = 2;
  if ((r = read_call_slot(ctx, O_VFF, v_ff, 0.))) return r;
  if ((r = read_call_slot(ctx, O_VCOUL, v_coul, ctx->C.charged ? 1. : 0.))) return r;
  if (v_ff)
    for (int k = 0; k < ctx->nrep; ++k) v_ff[k] += ctx->v_ff_walls[k];
  return MFA_OK;
}

int mfa_fluid_wall(mfa_ctx* ctx, int32_t wall_type, double* v_fw) {
  if (!ctx) return MFA_ERR_ARG;
  int r;
  if ((r = zero_call_slot(ctx, O_VFW)) || (r = zero_call_group(ctx, V_WALL))) return r;
  if (wall_type == 2 && ctx->C.wall == 2) {
    launch_wall(ctx->S, ctx->C, ctx->st, true, acc_of(ctx->acc_call, ctx->nrep));
    ctx->launches += 1;
  } else if (wall_type != 1) {
    return fail(ctx, MFA_ERR_UNSUPPORTED, "fluid_wall: only wall types 1 (in the pair kernel) and 2 are built");
  }
  CK(cudaGetLastError());
  return read_call_slot(ctx, O_VFW, v_fw, 0.);
}

int mfa_wall_wall(mfa_ctx* ctx, int32_t wall_type, double* v_ww) {
  if (!ctx) return MFA_ERR_ARG;
  if (v_ww)
    for (int k = 0; k < ctx->nrep; ++k) v_ww[k] = (wall_type == 2) ? ctx->v_ww[k] : 0.;
  return MFA_OK;
}

static int bonded_call(mfa_ctx* ctx, int mask, int slot, double* out) {
  int r;
  const int group = mask == 1 ? V_FENE : mask == 2 ? V_BEND : mask == 4 ? V_BENDM : V_OR;
  if ((r = zero_call_slot(ctx, slot)) || (r = zero_call_group(ctx, group))) return r;
  launch_bonded(ctx->S, ctx->C, ctx->st, mask, true, acc_of(ctx->acc_call, ctx->nrep));
  ctx->launches += 1;
  CK(cudaGetLastError());
  return read_call_slot(ctx, slot, out, 0.);
}

int mfa_intra_molec(mfa_ctx* ctx, double* v) { return ctx ? bonded_call(ctx, 1, O_VINTRA, v) : MFA_ERR_ARG; }
int mfa_bending(mfa_ctx* ctx, int32_t mode, double* v) {
  if (!ctx) return MFA_ERR_ARG;
  return mode == 0 ? MFA_OK : bonded_call(ctx, 2, O_VBEND, v);
}
int mfa_bending_melt(mfa_ctx* ctx, int32_t mode, double* v) {
  if (!ctx) return MFA_ERR_ARG;
  return mode == 0 ? MFA_OK : bonded_call(ctx, 4, O_VBENDM, v);
}
int mfa_orientation(mfa_ctx* ctx, int32_t mode, double* v) {
  if (!ctx) return MFA_ERR_ARG;
  return mode == 0 ? MFA_OK : bonded_call(ctx, 8, O_VOR, v);
}

int mfa_ewald_k(mfa_ctx* ctx, int32_t mode, double* v) {
  if (!ctx) return MFA_ERR_ARG;
  if (mode == 0) return MFA_OK;
  if (!ctx->kspace) return fail(ctx, MFA_ERR_STATE, "ewald_k: not a charged system");
  int r;
  if ((r = zero_call_slot(ctx, O_VCOULK)) || (r = zero_call_group(ctx, V_KSPACE))) return r;
  for (const KSpace& K : ctx->Ks) launch_kspace(ctx->S, ctx->C, K, ctx->st, true, acc_of(ctx->acc_call, ctx->nrep));
  ctx->launches += 4 * (long long)ctx->Ks.size();
  CK(cudaGetLastError());
  return read_call_slot(ctx, O_VCOULK, v, 0.);
}

int mfa_dipolar_correction(mfa_ctx* ctx, double* v) {
  if (!ctx) return MFA_ERR_ARG;
  if (!ctx->kspace) return fail(ctx, MFA_ERR_STATE, "dipolar_correction: not a charged system");
  int r;
  if ((r = zero_call_slot(ctx, O_VDIP)) || (r = zero_call_group(ctx, V_DIP))) return r;
  for (const KSpace& K : ctx->Ks) launch_dipolar(ctx->S, ctx->C, K, ctx->st, true, acc_of(ctx->acc_call, ctx->nrep));
  ctx->launches += 2 * (long long)ctx->Ks.size();
  CK(cudaGetLastError());
  return read_call_slot(ctx, O_VDIP, v, 0.);
}

int mfa_constant_force(mfa_ctx* ctx, int32_t mode) {
  if (!ctx) return MFA_ERR_ARG;
  if (mode != 1) return fail(ctx, MFA_ERR_UNSUPPORTED, "constant_force: only mode 1 (Poiseuille) is built");
  launch_const_force(ctx->S, ctx->C, ctx->st);
  ctx->launches += 1;
  CK(cudaGetLastError());
  return MFA_OK;
}

int mfa_verlet_velocities(mfa_ctx* ctx, mfa_energies* e) {
  if (!ctx) return MFA_ERR_ARG;
  int r;
  if ((r = zero_call_slot(ctx, O_TFLUID)) || (r = zero_call_slot(ctx, O_FH, 6)) || (r = zero_call_slot(ctx, O_KIN, 9)))
    return r;
  launch_integrate(ctx->S, ctx->C, ctx->st, 1, false, true, acc_of(ctx->acc_call, ctx->nrep));
  ctx->launches += 1;
  CK(cudaGetLastError());
  ctx->host_steps += 1;
  ctx->last_source = 2;
  if (e) {
    std::vector<double> h(NOBS * ctx->nrep);
    CK(cudaMemcpyAsync(h.data(), ctx->acc_call, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->st));
    RET(post_status(ctx));
    if ((r = check_status(ctx))) return r;
    for (int k = 0; k < ctx->nrep; ++k) fill_energies(ctx, h.data(), k, &e[k]);
  }
  return MFA_OK;
}

int mfa_profiles_accumulate(mfa_ctx* ctx) {
  if (!ctx) return MFA_ERR_ARG;
  launch_profiles(ctx->S, ctx->C, ctx->st, ctx->prof, ctx->C.hist_dim);
  ctx->launches += 1;
  ctx->n_obs += 1;
  CK(cudaGetLastError());
  return MFA_OK;
}

// ---- fused step -----------------------------------------------------------------------------
// Issues the kernels of `n` steps; eflag on steps where (absolute step) % energy_every == 0 and
// on the last step.  Returns the number of launches issued.
// Raises the neighbour-list capacity by half (at most NL_CAP_MAX), rebuilds the lists and drops
// the captured step graphs, which hold the old list address and capacity.
static int grow_lists(mfa_ctx* ctx) {
  ctx->grow_pending = false;
  DevState& S = ctx->S;
  const int seen = (int)ctx->h_status[1];
  const int newcap = std::min(NL_CAP_MAX, std::max(S.nbr_cap * 3 / 2, seen * 3 / 2 + 16));
  if (newcap <= S.nbr_cap) return MFA_OK;
  CK(cudaStreamSynchronize(ctx->st));
  auto it = std::find(ctx->allocs.begin(), ctx->allocs.end(), (void*)S.nbr);
  if (it != ctx->allocs.end()) { cudaFree(*it); ctx->allocs.erase(it); }
  S.nbr = nullptr;
  DA(S.nbr, (size_t)newcap * S.Np);
  S.nbr_cap = newcap;
  for (auto& g : ctx->graphs) cudaGraphExecDestroy(g.second.first);
  ctx->graphs.clear();
  // the overflow of the old capacity is over once the lists are rebuilt with the new one (the
  // rebuild sets the bit again if they still do not fit); the other status bits stay
  k_clear_overflow<<<1, 1, 0, ctx->st>>>(S.status);
  ctx->h_status[0] &= ~ST_NLIST_OVERFLOW;
  ctx->h_status[1] = 0;
  ctx->overflow_reported = false;
  rebuild(ctx, true);
  return MFA_OK;
}

// Start of mfa_step / mfa_verlet_positions: the status of earlier calls (when it has arrived)
// schedules a capacity growth; the growth runs before any new step.  An overflow seen here that no
// status-returning call has reported yet means that the steps since that rebuild ran on truncated
// lists: the capacity is raised, the lists rebuilt, and the call returns MFA_ERR_NLIST_OVERFLOW
// without running steps.  At the largest capacity an overflow cannot be repaired and is returned
// on every call.
static int prepare_step(mfa_ctx* ctx) {
  const int p = poll_status(ctx);
  if (p != MFA_OK && p != MFA_ERR_NLIST_OVERFLOW) return p;
  const bool over = p == MFA_ERR_NLIST_OVERFLOW;
  if (over && ctx->S.nbr_cap >= NL_CAP_MAX)
    return fail(ctx, MFA_ERR_NLIST_OVERFLOW,
                "neighbour lists overflow at the largest capacity (" + std::to_string(NL_CAP_MAX) + ")");
  const bool report = over && !ctx->overflow_reported;
  if (over) ctx->grow_pending = true;
  const int cap0 = ctx->S.nbr_cap;
  if (ctx->grow_pending) RET(grow_lists(ctx));
  if (report)
    return fail(ctx, MFA_ERR_NLIST_OVERFLOW,
                "neighbour lists of an earlier rebuild were truncated (capacity " + std::to_string(cap0) +
                    "); the steps since then used them; capacity now " + std::to_string(ctx->S.nbr_cap) +
                    " and the lists rebuilt");
  return MFA_OK;
}

// obs: the energy records also go into the observation averages (Rg^2 and momentum of the state
// of the record's step, so those steps run the velocity and position halves as two kernels).
// The context's state with the two view buffer sets (and step counters) exchanged.
static DevState other_views(const DevState& S) {
  DevState T = S;
  std::swap(T.pfx, T.pfx_alt);
  std::swap(T.vf, T.vf_alt);
  std::swap(T.steps_done, T.steps_alt);
  return T;
}

// n steps of the fused path (mfa_step).  With ctx->fuse_integ, a step without an energy record,
// profile or observation, other than the last, runs its integration in the pair kernel's tail,
// which writes the next step's views into the other buffer set: the sets alternate on each such
// step.  The chunk starts in the set that makes it end in the context's own (ctx->S): the first
// position update then copies the wall beads' views and the step counter across.
static long long issue_steps(mfa_ctx* ctx, int n, int phase, bool prof, bool obs, bool capturing, int* err) {
  const SimConst& C = ctx->C;
  cudaStream_t st = ctx->st;
  Acc acc = acc_of(ctx->acc_step, ctx->nrep);
  const int mask = any_chains(ctx) ? bonded_mask(ctx) : 0;
  long long L = 0;
  auto energies_at = [&](int k) { return ((phase + k) % ctx->opt.energy_every == 0) || k == n; };
  // (an energy step fuses too, unless it also observes: the observation reads the state after its
  // velocity update and before its position update)
  auto fused_at = [&](int k) { return ctx->fuse_integ && k < n && !prof && !(obs && energies_at(k)); };
  int n_fused = 0;
  for (int k = 1; k <= n; ++k) n_fused += fused_at(k) ? 1 : 0;
  const DevState sets[2] = {ctx->S, other_views(ctx->S)};
  int cur = n_fused & 1;
  {
    DevState S0 = sets[cur];
    S0.sync_alt = cur;
    launch_integrate(S0, C, st, 0, false, false, acc);
    L += 1;
  }
  for (int k = 1; k <= n; ++k) {
    const DevState& S = sets[cur];
    const bool ef = energies_at(k);
    DevState Sr = S;  // the step's rebuild leaves the (dead) accelerations of mobile particles behind
    Sr.permute_accel = 0;
    if (capturing) {
      int r = capture_conditional_rebuild(ctx, Sr);
      if (r != MFA_OK) {
        *err = r;
        return L;
      }
      L += 1;  // the rebuild body's launches are not counted: they run only when triggered
    } else {
      launch_rebuild(Sr, st, false);
      L += kRebuildLaunches;
    }
    const bool split = prof || (obs && ef);
    if (fused_at(k)) {  // forces and this step's integration in one kernel; the views move across
      launch_pair(S, C, st, false, ef, acc, ctx->opt.block_size, mask, true);
      L += 1;
      cur ^= 1;
    } else {
      // mixed: bonded terms inside the pair kernel; FP64: their own kernel
      launch_pair(S, C, st, false, ef, acc, ctx->opt.block_size, S.mixed ? mask : 0);
      L += 1;
      if (mask && !S.mixed) { launch_bonded(S, C, st, mask, ef, acc, true); L += 1; }
      if (ctx->kspace) {
        for (const KSpace& K : ctx->Ks) {
          launch_kspace(S, C, K, st, ef, acc, true);
          launch_dipolar(S, C, K, st, ef, acc, true);
          L += 7;
        }
      }
      if (k < n && !split) {
        launch_integrate(S, C, st, 2, true, ef, acc);
        L += 1;
      } else {
        launch_integrate(S, C, st, 1, true, ef, acc);
        L += 1;
        if (prof) { launch_profiles(S, C, st, ctx->prof, C.hist_dim); L += 1; }
      }
    }
    if (ef) {
      // the set that holds the step counter after this step's integration
      const DevState& Sn = sets[cur];
      launch_record(acc, ctx->rec, st);
      L += 1;
      if (obs) {
        launch_observe(Sn, C, st, ctx->obs);
        launch_obs_accum(Sn, C, st, ctx->rec, ctx->obs, ctx->avg);
        L += 2;
      }
      if (ctx->series) {
        launch_series(Sn, st, ctx->rec, ctx->series, ctx->series_step, ctx->series_head, ctx->opt.series_capacity);
        L += 2;
      }
    }
    if (split && k < n) {
      launch_integrate(S, C, st, 0, false, false, acc);
      L += 1;
    }
  }
  return L;
}

int mfa_list_stats(mfa_ctx* ctx, int32_t* capacity, int32_t* max_count) {
  if (!ctx) return MFA_ERR_ARG;
  RET(post_status(ctx));
  int r = check_status(ctx);
  if (capacity) *capacity = ctx->S.nbr_cap;
  if (max_count) *max_count = (int32_t)ctx->h_status[1];
  return r;
}

int mfa_get_options(mfa_ctx* ctx, mfa_options* out) {
  if (!ctx || !out) return MFA_ERR_ARG;
  *out = ctx->opt;
  out->list_cells = ctx->S.nl_h;
  out->list_cells_x = ctx->S.nl_hx;
  return MFA_OK;
}

int mfa_kspace_info_replica(mfa_ctx* ctx, int32_t rep, int32_t* n_k, int32_t* n_charged) {
  if (!ctx) return MFA_ERR_ARG;
  if (rep < 0 || rep >= ctx->nrep) return fail(ctx, MFA_ERR_ARG, "kspace_info_replica: no such replica");
  if (n_k) *n_k = ctx->kspace ? ctx->Ks[rep].nk : 0;
  if (n_charged) *n_charged = ctx->kspace ? ctx->Ks[rep].nq : 0;
  return MFA_OK;
}

int mfa_kspace_info(mfa_ctx* ctx, int32_t* n_k, int32_t* n_charged) {
  if (!ctx) return MFA_ERR_ARG;
  if (n_k) *n_k = ctx->kspace ? ctx->Ks[0].nk : 0;
  if (n_charged) *n_charged = ctx->kspace ? ctx->Ks[0].nq : 0;
  return MFA_OK;
}

int mfa_step(mfa_ctx* ctx, int32_t nsteps) {
  if (!ctx) return MFA_ERR_ARG;
  if (nsteps <= 0) return MFA_OK;
  RET(prepare_step(ctx));
  const long long s0 = ctx->sys[0].s_time + ctx->host_steps;
  const bool phased = ctx->P.flags.profiles || ctx->opt.observe;
  const bool observing = phased && ctx->host_steps >= ctx->opt.profile_from_step;
  if (phased && !observing && ctx->host_steps + nsteps > ctx->opt.profile_from_step) {
    // split at the start of the observation phase (md_main.f90:202)
    int first = (int)(ctx->opt.profile_from_step - ctx->host_steps);
    int r = mfa_step(ctx, first);
    if (r) return r;
    return mfa_step(ctx, nsteps - first);
  }
  const bool prof = ctx->P.flags.profiles && observing;
  const bool obs = ctx->opt.observe && observing;
  const int phase = (int)(s0 % ctx->opt.energy_every);
  long long L = 0;
  if (ctx->opt.use_graphs) {
    auto key = std::make_tuple(nsteps, phase, (int)prof, (int)obs);
    auto it = ctx->graphs.find(key);
    if (it == ctx->graphs.end()) {
      cudaGraph_t g;
      int err = MFA_OK;
      CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
      L = issue_steps(ctx, nsteps, phase, prof, obs, true, &err);
      cudaError_t ec = cudaStreamEndCapture(ctx->st, &g);
      if (err != MFA_OK) return err;
      CK(ec);
      cudaGraphExec_t ge;
      CK(cudaGraphInstantiate(&ge, g, 0));
      cudaGraphDestroy(g);
      it = ctx->graphs.emplace(key, std::make_pair(ge, L)).first;
    }
    CK(cudaGraphLaunch(it->second.first, ctx->st));
    L = it->second.second;
  } else {
    int err = MFA_OK;
    L = issue_steps(ctx, nsteps, phase, prof, obs, false, &err);
    CK(cudaGetLastError());
  }
  ctx->launches += L;
  ctx->host_steps += nsteps;
  if (prof) ctx->n_obs += nsteps;
  ctx->last_source = 1;
  return post_status(ctx);
}

int mfa_get_step(mfa_ctx* ctx, int64_t* step) {
  if (!ctx || !step) return MFA_ERR_ARG;
  *step = ctx->sys[0].s_time + ctx->host_steps;
  return MFA_OK;
}

// ---- data movement --------------------------------------------------------------------------
// The context's staging buffer for state movement (caller layout, 4 arrays of 3N doubles).
static int staging(mfa_ctx* ctx, double** out) {
  if (!ctx->stage) RET(dalloc(ctx, &ctx->stage, 12 * (size_t)ctx->N));
  *out = ctx->stage;
  return MFA_OK;
}

int mfa_sync_to_host(mfa_ctx* ctx, double* r0, double* v, double* a, double* force) {
  if (!ctx) return MFA_ERR_ARG;
  size_t n3 = 3 * (size_t)ctx->N;
  double* host[4] = {r0, v, a, force};
  if (!r0 && !v && !a && !force) return mfa_synchronize(ctx);
  double* buf = nullptr;
  RET(staging(ctx, &buf));
  // One array at a time: its gather into the staging buffer (device memory, the compute stream),
  // then its copy-engine copy to the host (the copy stream) while the next array is gathered.
  // (A gather kernel writing to host memory directly measured 3x slower than this.)
  for (int k = 0; k < 4; ++k) {
    if (!host[k]) continue;
    double* d = buf + k * n3;
    launch_gather_state(ctx->S, ctx->st, k == 0 ? d : nullptr, k == 1 ? d : nullptr, k == 2 ? d : nullptr,
                        k == 3 ? d : nullptr);
    CK(cudaEventRecord(ctx->ev_io[k], ctx->st));
    CK(cudaStreamWaitEvent(ctx->stc, ctx->ev_io[k], 0));
    CK(cudaMemcpyAsync(host[k], d, n3 * 8, cudaMemcpyDeviceToHost, ctx->stc));
  }
  CK(cudaEventRecord(ctx->ev_io[4], ctx->stc));
  CK(cudaStreamWaitEvent(ctx->st, ctx->ev_io[4], 0));
  RET(post_status(ctx));
  return check_status(ctx);
}

int mfa_set_state(mfa_ctx* ctx, const double* r0, const double* v, const double* a) {
  if (!ctx) return MFA_ERR_ARG;
  size_t n3 = 3 * (size_t)ctx->N;
  const double* host[3] = {r0, v, a};
  if (r0 || v || a) {
    double* buf = nullptr;
    RET(staging(ctx, &buf));
    // One array at a time: its copy-engine copy into the staging buffer (the copy stream, after
    // all earlier work of the context), then its scatter into slot order (the compute stream)
    // while the next array is copied.
    CK(cudaEventRecord(ctx->ev_io[4], ctx->st));
    CK(cudaStreamWaitEvent(ctx->stc, ctx->ev_io[4], 0));
    for (int k = 0; k < 3; ++k) {
      if (!host[k]) continue;
      CK(cudaMemcpyAsync(buf + k * n3, host[k], n3 * 8, cudaMemcpyHostToDevice, ctx->stc));
      CK(cudaEventRecord(ctx->ev_io[k], ctx->stc));
    }
    for (int k = 0; k < 3; ++k) {
      if (!host[k]) continue;
      const double* d = buf + k * n3;
      CK(cudaStreamWaitEvent(ctx->st, ctx->ev_io[k], 0));
      launch_scatter_state(ctx->S, ctx->st, k == 0 ? d : nullptr, k == 1 ? d : nullptr, k == 2 ? d : nullptr);
    }
  }
  // the lists stay valid unless some particle moved more than skin/2 from the last rebuild
  launch_refresh_views(ctx->S, ctx->C, ctx->st);
  rebuild(ctx, false);
  return mfa_synchronize(ctx);
}

int mfa_get_energies(mfa_ctx* ctx, mfa_energies* out) {
  if (!ctx || !out) return MFA_ERR_ARG;
  std::vector<double> h(NOBS * ctx->nrep);
  const double* src = ctx->last_source == 2 ? ctx->acc_call : ctx->rec;
  CK(cudaMemcpyAsync(h.data(), src, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->st));
  RET(post_status(ctx));
  int r = check_status(ctx);
  if (r) return r;
  for (int k = 0; k < ctx->nrep; ++k) fill_energies(ctx, h.data(), k, &out[k]);
  return MFA_OK;
}

int mfa_get_averages(mfa_ctx* ctx, mfa_averages* out) {
  if (!ctx || !out) return MFA_ERR_ARG;
  if (!ctx->avg) return fail(ctx, MFA_ERR_STATE, "observation averages need options.observe = 1");
  const int R = ctx->nrep;
  std::vector<double> h((size_t)NAVG * R);
  CK(cudaMemcpyAsync(h.data(), ctx->avg, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->st));
  RET(post_status(ctx));
  int r = check_status(ctx);
  if (r) return r;
  for (int k = 0; k < R; ++k) {
    const double* a = &h[(size_t)NAVG * k];
    mfa_averages& o = out[k];
    std::memset(&o, 0, sizeof o);
    o.count = (int64_t)a[A_COUNT];
    if (o.count == 0) continue;
    const double ic = 1. / a[A_COUNT];
    o.v_total = a[A_VT] * ic; o.t_total = a[A_TT] * ic; o.e_total = a[A_ET] * ic;
    o.v_total2 = a[A_VT2] * ic; o.t_total2 = a[A_TT2] * ic; o.e_total2 = a[A_ET2] * ic;
    o.v_fluid = a[A_VF] * ic; o.t_fluid = a[A_TF] * ic; o.e_fluid = a[A_EF] * ic;
    o.v_fluid2 = a[A_VF2] * ic; o.t_fluid2 = a[A_TF2] * ic; o.e_fluid2 = a[A_EF2] * ic;
    for (int d = 0; d < 3; ++d) {
      o.momentum[d] = a[A_MOM + d] * ic;
      o.rg2_brush[d] = a[A_RGB + d] * ic;
      o.rg2_melt[d] = a[A_RGM + d] * ic;
      o.rg2_mean[d] = a[A_RGA + d] * ic;
    }
    o.r_par_per2[0] = a[A_RPP] * ic;
    o.r_par_per2[1] = a[A_RPP + 1] * ic;
    for (int c = 0; c < 9; ++c) o.pressure[c] = a[A_P + c] * ic;
    for (int c = 0; c < 6; ++c) o.f_heads[c / 3][c % 3] = a[A_FH + c] * ic;
  }
  return MFA_OK;
}

int mfa_reset_averages(mfa_ctx* ctx) {
  if (!ctx) return MFA_ERR_ARG;
  if (ctx->avg) CK(cudaMemsetAsync(ctx->avg, 0, sizeof(double) * NAVG * ctx->nrep, ctx->st));
  return MFA_OK;
}

int mfa_get_energy_series(mfa_ctx* ctx, mfa_energies* out, int32_t cap, int32_t* n) {
  if (!ctx || !n || cap < 0 || (cap > 0 && !out)) return MFA_ERR_ARG;
  *n = 0;
  if (!ctx->series) return fail(ctx, MFA_ERR_STATE, "the energy series needs options.series_capacity > 0");
  long long head = 0;
  CK(cudaMemcpyAsync(&head, ctx->series_head, sizeof head, cudaMemcpyDeviceToHost, ctx->st));
  RET(post_status(ctx));
  int r = check_status(ctx);
  if (r) return r;
  const int R = ctx->nrep, scap = ctx->opt.series_capacity;
  long long first = std::max(ctx->series_read, head - scap);  // the oldest record still in the ring
  const long long cnt = std::min<long long>(head - first, cap);
  std::vector<double> rec((size_t)O_VIR * R, 0.), acc((size_t)NOBS * R, 0.);
  for (long long k = 0; k < cnt; ++k) {
    const int slot = (int)((first + k) % scap);
    long long sd = 0;
    CK(cudaMemcpy(rec.data(), ctx->series + (size_t)slot * O_VIR * R, sizeof(double) * rec.size(),
                  cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&sd, ctx->series_step + slot, sizeof sd, cudaMemcpyDeviceToHost));
    std::copy(rec.begin(), rec.end(), acc.begin());
    for (int q = 0; q < R; ++q) {
      mfa_energies& e = out[k * R + q];
      record_energies(acc.data(), R, q, ctx->hreps[q], ctx->C, &e);
      e.step = ctx->sys[q].s_time + sd;
    }
  }
  ctx->series_read = first + cnt;
  *n = (int32_t)cnt;
  return MFA_OK;
}

int mfa_get_virial(mfa_ctx* ctx, mfa_virial* out) {
  if (!ctx || !out) return MFA_ERR_ARG;
  std::vector<double> h(NOBS * ctx->nrep);
  const double* src = ctx->last_source == 2 ? ctx->acc_call : ctx->rec;
  CK(cudaMemcpyAsync(h.data(), src, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->st));
  RET(post_status(ctx));
  int r = check_status(ctx);
  if (r) return r;
  for (int k = 0; k < ctx->nrep; ++k) fill_virial(ctx, h.data(), k, &out[k]);
  return MFA_OK;
}

int mfa_observe(mfa_ctx* ctx, mfa_observables* out) {
  if (!ctx || !out) return MFA_ERR_ARG;
  const int R = ctx->nrep;
  launch_observe(ctx->S, ctx->C, ctx->st, ctx->obs);
  ctx->launches += 1;
  std::vector<double> h((size_t)9 * R), a((size_t)NOBS * R);
  CK(cudaMemcpyAsync(h.data(), ctx->obs, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->st));
  const double* src = ctx->last_source == 2 ? ctx->acc_call : ctx->rec;
  CK(cudaMemcpyAsync(a.data(), src, sizeof(double) * a.size(), cudaMemcpyDeviceToHost, ctx->st));
  RET(post_status(ctx));
  int r = check_status(ctx);
  if (r) return r;
  for (int k = 0; k < R; ++k) {
    mfa_observables& o = out[k];
    std::memset(&o, 0, sizeof o);
    o.step = ctx->sys[k].s_time + ctx->host_steps;
    for (int d = 0; d < 3; ++d) {
      o.rg2_brush[d] = h[(size_t)9 * k + d];
      o.rg2_melt[d] = h[(size_t)9 * k + 3 + d];
      o.momentum[d] = h[(size_t)9 * k + 6 + d];
      o.f_heads[0][d] = a[(size_t)(O_FH + d) * R + k];
      o.f_heads[1][d] = a[(size_t)(O_FH + 3 + d) * R + k];
    }
  }
  return MFA_OK;
}

int mfa_get_profiles(mfa_ctx* ctx, int32_t rep, double* dens, double* vsum, double* v2sum, int64_t* n_obs) {
  if (!ctx || rep < 0 || rep >= ctx->nrep) return MFA_ERR_ARG;
  const int H = ctx->C.hist_dim;
  std::vector<double> h((size_t)H * 21);
  CK(cudaMemcpyAsync(h.data(), ctx->prof + (size_t)rep * H * 21, sizeof(double) * h.size(), cudaMemcpyDeviceToHost,
                     ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  for (int b = 0; b < H; ++b)
    for (int sp = 0; sp < 3; ++sp) {
      const double* q = &h[(b * 3 + sp) * 7];
      if (dens) dens[b * 3 + sp] = q[0];
      for (int d = 0; d < 3; ++d) {
        if (vsum) vsum[(b * 3 + sp) * 3 + d] = q[1 + d];
        if (v2sum) v2sum[(b * 3 + sp) * 3 + d] = q[4 + d];
      }
    }
  if (n_obs) *n_obs = ctx->n_obs;
  return MFA_OK;
}

int mfa_reset_profiles(mfa_ctx* ctx) {
  if (!ctx) return MFA_ERR_ARG;
  CK(cudaMemsetAsync(ctx->prof, 0, sizeof(double) * ctx->nrep * ctx->C.hist_dim * 21, ctx->st));
  ctx->n_obs = 0;
  return MFA_OK;
}

// ---- parity exports -------------------------------------------------------------------------
int mfa_cell_list(mfa_ctx* ctx, int32_t rep, int32_t l_box, int32_t* cell_of, int32_t* counts, int32_t counts_cap,
                  int32_t* n_cells) {
  if (!ctx || rep < 0 || rep >= ctx->nrep || !cell_of || !n_cells || (l_box != 1 && l_box != 2)) return MFA_ERR_ARG;
  const mfa_system& s = ctx->sys[rep];
  const double rc = ctx->P.r_cut_max;
  int nc[3];
  double il[3];
  for (int d = 0; d < 3; ++d) {  // make_binning (cell_list.f90:137-151)
    nc[d] = (l_box == 1) ? (int)(s.boundary[d] / rc) : (int)(s.boundary[d] / (rc / 2.));
    if (nc[d] < 1) nc[d] = 1;
    double l = s.boundary[d] / (double)(float)nc[d];
    il[d] = 1 / l;
    n_cells[d] = nc[d];
  }
  const int nct = nc[0] * nc[1] * nc[2];
  if (counts && counts_cap < nct + 1) return fail(ctx, MFA_ERR_CAPACITY, "counts_cap < n_cells_tot + 1");
  int *dco = nullptr, *dcnt = nullptr;
  CK(cudaMallocAsync(&dco, sizeof(int) * std::max(1, s.n_mon_tot), ctx->st));
  CK(cudaMallocAsync(&dcnt, sizeof(int) * (nct + 1), ctx->st));
  CK(cudaMemsetAsync(dcnt, 0, sizeof(int) * (nct + 1), ctx->st));
  launch_ref_cells(ctx->S, ctx->st, rep, il, nc, dco, dcnt);
  ctx->launches += 1;
  CK(cudaMemcpyAsync(cell_of, dco, sizeof(int) * s.n_mon_tot, cudaMemcpyDeviceToHost, ctx->st));
  if (counts) CK(cudaMemcpyAsync(counts, dcnt, sizeof(int) * (nct + 1), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaFreeAsync(dco, ctx->st));
  CK(cudaFreeAsync(dcnt, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return MFA_OK;
}

int mfa_cell_neigh_list(const int32_t* n_cells, int32_t n_nei, int32_t* out) {
  if (!n_cells || !out || (n_nei != 13 && n_nei != 62)) return MFA_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MFA_ERR_NO_DEVICE;
  const long long nct = (long long)n_cells[0] * n_cells[1] * n_cells[2];
  if (nct <= 0 || nct > (1ll << 26)) return MFA_ERR_ARG;
  int* d = nullptr;
  if (cudaMalloc(&d, sizeof(int) * nct * n_nei) != cudaSuccess) return MFA_ERR_ALLOC;
  launch_cell_neigh(n_cells, n_nei, d, 0);
  cudaError_t e = cudaMemcpy(out, d, sizeof(int) * nct * n_nei, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? MFA_OK : MFA_ERR_CUDA;
}

int mfa_pair_list(mfa_ctx* ctx, int32_t rep, int32_t* pairs, int64_t cap, int64_t* n) {
  if (!ctx || rep < 0 || rep >= ctx->nrep || !n || cap < 0) return MFA_ERR_ARG;
  int* dp = nullptr;
  unsigned long long* dc = nullptr;
  cudaError_t ea = cudaMallocAsync(&dp, sizeof(int) * 2 * std::max<int64_t>(cap, 1), ctx->st);
  if (ea == cudaSuccess) {
    ea = cudaMallocAsync(&dc, sizeof(unsigned long long), ctx->st);
    if (ea != cudaSuccess) cudaFreeAsync(dp, ctx->st);
  }
  if (ea != cudaSuccess) {
    cudaGetLastError();  // not sticky: later launch checks must not see it
    return fail(ctx, MFA_ERR_ALLOC, std::string("pair-list scratch (cudaMallocAsync): ") + cudaGetErrorString(ea) +
                                        "; mfa_pair_list_static takes no device memory");
  }
  CK(cudaMemsetAsync(dc, 0, sizeof(unsigned long long), ctx->st));
  launch_pair_list(ctx->S, ctx->C, ctx->st, rep, dp, cap, dc);
  ctx->launches += 1;
  unsigned long long hc = 0;
  CK(cudaMemcpyAsync(&hc, dc, sizeof hc, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  *n = (int64_t)hc;
  if (pairs && cap > 0)
    CK(cudaMemcpyAsync(pairs, dp, sizeof(int) * 2 * std::min<int64_t>(cap, (int64_t)hc), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaFreeAsync(dp, ctx->st));
  CK(cudaFreeAsync(dc, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return MFA_OK;
}

// ---- mfa_pair_list without device allocation -----------------------------------------------
// Same result as mfa_pair_list, staged in file-scope device arrays instead of memory taken from
// the allocator: MFA_PAIR_LIST_STATIC_MAX pairs and one counter.  The driver places them on each
// device when it loads this module; every device that loads the library holds them until exit.
// Host code must not hand the array names to a kernel (on the host they are stand-ins, not device
// addresses): their device addresses are looked up with cudaGetSymbolAddress at the first call on
// a context, with the context's device current, and kept in the context.  That first call may load
// the module, so it must come before any stream capture.  A context made after a device reset
// looks them up again.  Every call shares the same scratch and finds the last call's contents in
// it: the counter is cleared on each call, and two calls that overlap on one device race.
static __device__ __align__(256) int g_static_pairs[2 * MFA_PAIR_LIST_STATIC_MAX];
static __device__ __align__(256) unsigned long long g_static_count;

static int pair_list_static_on_device(mfa_ctx* ctx, int32_t rep, int32_t* pairs, int64_t cap, int64_t* n) {
  if (!ctx->static_pairs) {
    void* a = nullptr;
    void* b = nullptr;
    CK(cudaGetSymbolAddress(&a, g_static_pairs));
    CK(cudaGetSymbolAddress(&b, g_static_count));
    ctx->static_pairs = static_cast<int*>(a);
    ctx->static_count = static_cast<unsigned long long*>(b);
  }
  int* dp = ctx->static_pairs;
  unsigned long long* dc = ctx->static_count;
  CK(cudaMemsetAsync(dc, 0, sizeof(unsigned long long), ctx->st));  // the pair counter starts at zero
  launch_pair_list(ctx->S, ctx->C, ctx->st, rep, dp, cap, dc);
  ctx->launches += 1;
  unsigned long long hc = 0;
  CK(cudaMemcpyAsync(&hc, dc, sizeof hc, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  *n = (int64_t)hc;
  if (pairs && cap > 0) {
    CK(cudaMemcpyAsync(pairs, dp, sizeof(int) * 2 * std::min<int64_t>(cap, (int64_t)hc), cudaMemcpyDeviceToHost,
                       ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
  }
  return MFA_OK;
}

int mfa_pair_list_static(mfa_ctx* ctx, int32_t rep, int32_t* pairs, int64_t cap, int64_t* n) {
  if (!ctx || rep < 0 || rep >= ctx->nrep || !n || cap < 0) return MFA_ERR_ARG;
  if (cap > MFA_PAIR_LIST_STATIC_MAX)
    return fail(ctx, MFA_ERR_CAPACITY,
                "cap above MFA_PAIR_LIST_STATIC_MAX (" + std::to_string(MFA_PAIR_LIST_STATIC_MAX) +
                    " pairs): use mfa_pair_list");
  // the context's device is made current for the call; the caller's current device is restored
  int prev = 0;
  CK(cudaGetDevice(&prev));
  if (prev != ctx->device) CK(cudaSetDevice(ctx->device));
  const int rc = pair_list_static_on_device(ctx, rep, pairs, cap, n);
  if (prev != ctx->device) {
    const cudaError_t e = cudaSetDevice(prev);
    if (rc == MFA_OK && e != cudaSuccess)
      return fail(ctx, MFA_ERR_CUDA, std::string("cudaSetDevice (restoring the caller's device): ") +
                                         cudaGetErrorString(e));
  }
  return rc;
}

// ---- timing ---------------------------------------------------------------------------------
int mfa_event_record(mfa_ctx* ctx, int32_t slot) {
  if (!ctx || slot < 0 || slot >= 16) return MFA_ERR_ARG;
  CK(cudaEventRecord(ctx->ev[slot], ctx->st));
  return MFA_OK;
}

int mfa_event_elapsed(mfa_ctx* ctx, int32_t a, int32_t b, float* ms) {
  if (!ctx || !ms || a < 0 || b < 0 || a >= 16 || b >= 16) return MFA_ERR_ARG;
  CK(cudaEventSynchronize(ctx->ev[b]));
  CK(cudaEventElapsedTime(ms, ctx->ev[a], ctx->ev[b]));
  return MFA_OK;
}

const char* mfa_kernel_name(int32_t fam) { return (fam >= 0 && fam < MFA_NKFAM) ? kFamNames[fam] : "?"; }

int mfa_kernel_times(mfa_ctx* ctx, int32_t nsteps, float* mean_ms, int32_t* launches) {
  if (!ctx || nsteps < 1 || !mean_ms) return MFA_ERR_ARG;
  const DevState& S = ctx->S;
  const SimConst& C = ctx->C;
  cudaStream_t st = ctx->st;
  Acc acc = acc_of(ctx->acc_step, ctx->nrep);
  const int mask = any_chains(ctx) ? bonded_mask(ctx) : 0;
  std::vector<cudaEvent_t> evs;
  std::vector<int> fam;
  auto mark = [&](int f) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, st);
    evs.push_back(e);
    fam.push_back(f);
  };
  // the first position update belongs to the "positions" family; each step then runs
  // rebuild, pair, bonded, kspace and the fused velocity+position kernel, as mfa_step runs them:
  // with ctx->fuse_integ the steps before the last (the energy step) integrate in the pair
  // kernel's tail, whose time then counts as "pair"
  const int n_fused = ctx->fuse_integ ? nsteps - 1 : 0;
  const DevState sets[2] = {S, other_views(S)};
  int cur = n_fused & 1;
  mark(-1);
  {
    DevState S0 = sets[cur];
    S0.sync_alt = cur;
    launch_integrate(S0, C, st, 0, false, false, acc);
  }
  mark(7);
  for (int k = 1; k <= nsteps; ++k) {
    const bool ef = (k == nsteps);
    const DevState& Sk = sets[cur];
    // the rebuild as the fused step runs it: the replicas whose skin test fired, if any
    DevState Sr = Sk;
    Sr.permute_accel = 0;
    launch_rebuild(Sr, st, false);
    mark(0);
    if (ctx->fuse_integ && !ef) {
      launch_pair(Sk, C, st, false, false, acc, ctx->opt.block_size, mask, true);
      mark(1);
      cur ^= 1;
      continue;
    }
    launch_pair(Sk, C, st, false, ef, acc, ctx->opt.block_size, S.mixed ? mask : 0);
    mark(1);
    if (mask && !S.mixed) { launch_bonded(Sk, C, st, mask, ef, acc, true); mark(2); }
    if (ctx->kspace) {
      for (const KSpace& K : ctx->Ks) {
        launch_kspace(Sk, C, K, st, ef, acc, true);
        launch_dipolar(Sk, C, K, st, ef, acc, true);
      }
      mark(4);
    }
    launch_integrate(Sk, C, st, k < nsteps ? 2 : 1, true, ef, acc);
    mark(3);
    if (ef) { launch_record(acc, ctx->rec, st); mark(6); }
  }
  // then a rebuild of every replica, three times
  for (int k = 0; k < 3; ++k) {
    launch_rebuild(S, st, true);
    mark(8);
  }
  CK(cudaStreamSynchronize(st));
  std::vector<double> tot(MFA_NKFAM, 0.);
  std::vector<int> cnt(MFA_NKFAM, 0);
  for (size_t k = 1; k < evs.size(); ++k) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, evs[k - 1], evs[k]);
    tot[fam[k]] += ms;
    cnt[fam[k]] += 1;
  }
  for (auto e : evs) cudaEventDestroy(e);
  for (int f = 0; f < MFA_NKFAM; ++f) {
    mean_ms[f] = cnt[f] ? (float)(tot[f] / cnt[f]) : 0.f;
    if (launches) launches[f] = cnt[f];
  }
  ctx->host_steps += nsteps;
  ctx->last_source = 1;
  return post_status(ctx);
}

int mfa_launch_count(mfa_ctx* ctx, int64_t* n) {
  if (!ctx || !n) return MFA_ERR_ARG;
  *n = ctx->launches;
  return MFA_OK;
}

int mfa_replica_rebuild_counts(mfa_ctx* ctx, int64_t* counts) {
  if (!ctx || !counts) return MFA_ERR_ARG;
  CK(cudaMemcpyAsync(counts, ctx->S.rep_rebuilds, sizeof(long long) * ctx->nrep, cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  return MFA_OK;
}

int mfa_rebuild_count(mfa_ctx* ctx, int64_t* n) {
  if (!ctx || !n) return MFA_ERR_ARG;
  CK(cudaMemcpyAsync(ctx->h_rebuilds, ctx->S.rebuilds, sizeof(long long), cudaMemcpyDeviceToHost, ctx->st));
  CK(cudaStreamSynchronize(ctx->st));
  *n = *ctx->h_rebuilds;
  return MFA_OK;
}

}  // extern "C"
