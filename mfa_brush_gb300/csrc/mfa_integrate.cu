// mfa_integrate.cu -- velocity-Verlet integration, profiles and host-layout kernels.
//
// k_integrate<MODE>:
//   MODE 0  verlet_positions.f90:150-209: r += dt v + dt^2/2 a, x,y wrapped into [0,L),
//           v += dt/2 a; then the pair-kernel views and the skin test (displacement since the
//           last rebuild > skin/2 raises the rebuild flag; check_skin.f90:11-24).
//   MODE 1  verlet_velocities.f90:25-153: a = F/m, v += dt/2 a, brush heads driven: a = F = 0
//           and v = (+-va_wall, 0) for the chains of the first / second half (:111-124, the two
//           brushes sheared against each other; va_wall = 0 without shear and always with
//           POISEUILLE, :113-120), kinetic energy.
//   MODE 2  MODE 1 of step n followed by MODE 0 of step n+1 in one pass (the fused step): one
//           read of r, v, F and one write of r, v and the views per particle per step.
//   add_ext adds the 9-3 wall force (fluid_wall.f90:96-121) and the body force
//           (constant_force.f90:17-21) inside the kernel instead of separate passes (FP64 step;
//           the mixed step adds them in the pair kernel).  With energies: the kinetic energy and
//           the kinetic tensor sum m v (x) v (viscosity.f90:20-27) of v(n).
// All integration is FP64 in both precision modes.
#include "mfa_obs.cuh"
#include "mfa_integ.cuh"

namespace mfa {

__device__ __forceinline__ void store_views(const DevState& s, int i, const RepDesc& R, double x, double y,
                                            double z, double vx, double vy, double vz, int w, int t, int4& q) {
  q.x = to_fx_periodic(x, R.sfx[0]);
  q.y = to_fx_periodic(y, R.sfx[1]);
  q.z = to_fx_z(z, R.sfx[2]);
  q.w = w;
  if (s.mixed) {
    s.pfx[i] = q;
    s.vf[i] = make_float4((float)vx, (float)vy, (float)vz, __int_as_float(t));
  } else {
    s.pd[i] = mk_dbl4(x, y, z, __longlong_as_double((long long)w));
    s.vd[i] = mk_dbl4(vx, vy, vz, __longlong_as_double((long long)t));
  }
}

template <int MODE, bool ADDEXT, bool EFLAG>
__global__ void __launch_bounds__(256) k_integrate(DevState s, SimConst C, Acc acc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool inside = i < s.N;
  const int w = inside ? s.info[i] : 0;
  const bool mob = inside && info_mobile(w);
  const int rep = info_rep(w);
  double ke = 0., efw = 0., wzz = 0.;
  double kin[6] = {0., 0., 0., 0., 0., 0.};  // m v (x) v: xx yy zz xy xz yz
  double fh[6] = {0., 0., 0., 0., 0., 0.};  // minus the head force, by half of the chains
  if (mob) {
    const RepDesc& R = s.reps[rep];
    const int t = info_type(w);
    double x = s.rx[i], y = s.ry[i], z = s.rz[i];
    double vx = s.vx[i], vy = s.vy[i], vz = s.vz[i];
    double ax, ay, az;
    if (MODE >= 1) {
      double Fx = s.fx[i], Fy = s.fy[i], Fz = s.fz[i];
      if (ADDEXT) {
        if (C.wall == 2) {
          double e, fb, ft;
          wall93_split(C, t, z, R.L[2], fb, ft, e);
          Fz += fb + ft;
          efw = e;
          wzz = fb * z + ft * (z - R.L[2]);  // each wall's force times z - z_wall
        }
        if (C.poiseuille && t != 0) {
          const double m = C.mass[t];
          Fx += m * C.const_force[0];
          Fy += m * C.const_force[1];
          Fz += m * C.const_force[2];
        }
      }
      const double im = C.inv_mass[t];
      ax = Fx * im; ay = Fy * im; az = Fz * im;
      vx = vx + C.half_dt * ax;
      vy = vy + C.half_dt * ay;
      vz = vz + C.half_dt * az;
      if (info_head(w)) {
        const bool first = (s.tag[i] - R.p0) / R.n_mon < R.n_chain / 2;
        if (EFLAG) {  // f_on_heads before the heads are held (verlet_velocities.f90:18)
          const int h = first ? 0 : 3;
          fh[h] = -Fx; fh[h + 1] = -Fy; fh[h + 2] = -Fz;
        }
        // verlet_velocities.f90:111-124: the heads move with their wall (+-va_wall in x, y)
        const double sg = first ? 1. : -1.;
        vx = sg * C.va_wall[0];
        vy = sg * C.va_wall[1];
        vz = 0.;
        ax = ay = az = 0.;
        if (MODE == 1) { s.fx[i] = 0.; s.fy[i] = 0.; s.fz[i] = 0.; }
      }
      if (EFLAG) {
        ke = 0.5 * C.mass[t] * (vx * vx + vy * vy + vz * vz);
        sym_add(kin, C.mass[t], vx, vy, vz);
      }
      if (MODE == 1) {
        s.ax[i] = ax; s.ay[i] = ay; s.az[i] = az;
        s.vx[i] = vx; s.vy[i] = vy; s.vz[i] = vz;
      }
    } else {
      ax = s.ax[i]; ay = s.ay[i]; az = s.az[i];
    }
    if (MODE == 0 || MODE == 2) {
      x = x + C.dt * vx + C.half_dt2 * ax;
      y = y + C.dt * vy + C.half_dt2 * ay;
      z = z + C.dt * vz + C.half_dt2 * az;
      if (x > R.L[0]) x -= R.L[0]; else if (x < 0.) x += R.L[0];
      if (y > R.L[1]) y -= R.L[1]; else if (y < 0.) y += R.L[1];
      vx = vx + C.half_dt * ax;
      vy = vy + C.half_dt * ay;
      vz = vz + C.half_dt * az;
      s.rx[i] = x; s.ry[i] = y; s.rz[i] = z;
      s.vx[i] = vx; s.vy[i] = vy; s.vz[i] = vz;
      int4 q;
      store_views(s, i, R, x, y, z, vx, vy, vz, w, s.tag[i], q);
      const int4 q0 = s.ref[i];
      const float dx = i2f_fast(fx_diff(q.x, q0.x)) * R.ufx_f[0];
      const float dy = i2f_fast(fx_diff(q.y, q0.y)) * R.ufx_f[1];
      const float dz = i2f_fast(fx_diff(q.z, q0.z)) * R.ufx_f[2];
      if (dx * dx + dy * dy + dz * dz > C.skin_half2_f) flag_rebuild(s, rep);
      if (!(isfinite(x) && isfinite(y) && isfinite(z))) atomicOr(s.status, ST_NAN);
    }
  } else if ((MODE == 0 || MODE == 2) && inside && C.move_walls) {  // a wall bead on a moving wall
    double x, y, z;
    int4 q = move_wall_bead(s, C, i, w, x, y, z);
    store_views(s, i, s.reps[rep], x, y, z, 0., 0., 0., w, s.tag[i], q);
  }
  if (MODE >= 1 && i == 0) *s.steps_done += 1;
  if (EFLAG && MODE >= 1) {
    int sl[15];
    double v[15];
    sl[0] = O_TFLUID; v[0] = ke;
    const int idx[6] = {0, 4, 8, 1, 2, 5};
    for (int c = 0; c < 6; ++c) {
      sl[1 + c] = O_KIN + idx[c]; v[1 + c] = kin[c];
      sl[7 + c] = O_FH + c; v[7 + c] = fh[c];
    }
    sl[13] = O_VFW; v[13] = efw;  // zero unless ADDEXT with implicit walls
    sl[14] = O_VIR + 9 * V_WALL + 8; v[14] = wzz;
    obs_push<double, 15>(acc, sl, v, rep, mob);
  }
}


// The integrator of the mixed-precision path with the FP64 work cut to the state accumulators
// (GB300 issues FP64 and every conversion instruction at 2 per SM per clock, 1/64 of FP32):
//   MODE 0  positions (verlet_positions): dv = dt/2 a(n-1); v += dv; r += dt v.
//   MODE 1  velocities (verlet_velocities): a = F/m; v += dt/2 a; heads fixed; a and the total
//           force are stored; kinetic energy.
//   MODE 2  both at once: v(n-1/2) -> v(n+1/2) with one FP64 add of dt a(n), r += dt v(n+1/2),
//           equal in exact arithmetic to MODE 1 followed by MODE 0; kinetic energy from
//           v(n) = v(n+1/2) - dt/2 a.
// r + dt v + dt^2/2 a is formed as r + dt (v + dt/2 a).  Accelerations and velocity increments
// are FP32; r and v stay FP64.  FUSED reads the force of the fused step (the pair kernel's total,
// walls and body force included, rounded to FP32); otherwise the FP64 force array of the
// per-routine path.  Conversions use the integer forms of mfa_dev.cuh.
template <int MODE, bool EFLAG, bool FUSED>
__global__ void __launch_bounds__(256) k_int_mixed(DevState s, SimConst C, Acc acc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool inside = i < s.N;
  const int w = inside ? s.info[i] : 0;
  const bool mob = inside && info_mobile(w);
  const int rep = info_rep(w);
  float ke = 0.f;
  float kin[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // m v (x) v: xx yy zz xy xz yz
  float fh[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // minus the head force, by half of the chains
  if (mob) {
    float Fx = 0.f, Fy = 0.f, Fz = 0.f;
    if (MODE >= 1) {
      if (FUSED) {
        const float4 F4 = s.f4[i];
        Fx = F4.x; Fy = F4.y; Fz = F4.z;
      } else {
        Fx = d2f_fast(s.fx[i]); Fy = d2f_fast(s.fy[i]); Fz = d2f_fast(s.fz[i]);
      }
    }
    int_mixed_particle<MODE, EFLAG>(s, C, i, w, Fx, Fy, Fz, s.pfx, s.vf, ke, kin, fh);
  } else if ((MODE == 0 || MODE == 2) && inside && C.move_walls) {  // a wall bead on a moving wall
    double x, y, z;
    s.pfx[i] = move_wall_bead(s, C, i, w, x, y, z);
    if (MODE == 0 && s.sync_alt) s.vf[i] = s.vf_alt[i];
  } else if (MODE == 0 && inside && s.sync_alt) {
    s.pfx[i] = s.pfx_alt[i];  // a chunk that starts in the other view buffers: the wall beads' views
    s.vf[i] = s.vf_alt[i];
  }
  if (MODE == 0 && s.sync_alt && i == 0) *s.steps_done = *s.steps_alt;
  if (MODE >= 1 && i == 0) *s.steps_done += 1;
  if (EFLAG && MODE >= 1) {
    int sl[13];
    float v[13];
    sl[0] = O_TFLUID; v[0] = ke;
    const int idx[6] = {0, 4, 8, 1, 2, 5};
    for (int c = 0; c < 6; ++c) {
      sl[1 + c] = O_KIN + idx[c]; v[1 + c] = kin[c];
      sl[7 + c] = O_FH + c; v[7 + c] = fh[c];
    }
    obs_push<float, 13>(acc, sl, v, rep, mob);
  }
}

template <int MODE>
static void launch_mode(const DevState& s, const SimConst& C, cudaStream_t st, bool add_ext, bool eflag, Acc acc) {
  const int B = 256, g = (s.N + B - 1) / B;
  if (s.mixed) {
    if (MODE == 0) k_int_mixed<0, false, false><<<g, B, 0, st>>>(s, C, acc);
    else if (add_ext && eflag) k_int_mixed<MODE, true, true><<<g, B, 0, st>>>(s, C, acc);
    else if (add_ext) k_int_mixed<MODE, false, true><<<g, B, 0, st>>>(s, C, acc);
    else if (eflag) k_int_mixed<MODE, true, false><<<g, B, 0, st>>>(s, C, acc);
    else k_int_mixed<MODE, false, false><<<g, B, 0, st>>>(s, C, acc);
    return;
  }
  if (add_ext) {
    if (eflag) k_integrate<MODE, true, true><<<g, B, 0, st>>>(s, C, acc);
    else k_integrate<MODE, true, false><<<g, B, 0, st>>>(s, C, acc);
  } else {
    if (eflag) k_integrate<MODE, false, true><<<g, B, 0, st>>>(s, C, acc);
    else k_integrate<MODE, false, false><<<g, B, 0, st>>>(s, C, acc);
  }
}

void launch_integrate(const DevState& s, const SimConst& C, cudaStream_t st, int mode, bool add_ext, bool eflag,
                      Acc acc) {
  if (mode == 0) launch_mode<0>(s, C, st, false, false, acc);
  else if (mode == 1) launch_mode<1>(s, C, st, add_ext, eflag, acc);
  else launch_mode<2>(s, C, st, add_ext, eflag, acc);
}

// ---------------------------------------------------------------------------------------------
// Profiles: histo(2) + velocity_prof(2) (functions.f90:157-214, 319-365).  Each block takes a
// contiguous run of slots, accumulates [bin][species][count, sum v, sum v^2] in shared memory
// and flushes to the replica's global FP64 profile whenever the replica changes.
// prof layout per replica: [hist][3 species][7] (count, vx, vy, vz, vx^2, vy^2, vz^2).
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_profiles(DevState s, SimConst C, double* __restrict__ prof, int H,
                                                  int chunk) {
  extern __shared__ double sh[];
  const int n_sh = H * 3 * 7;
  const int b0 = blockIdx.x * chunk, b1 = min(s.N, b0 + chunk);
  if (b0 >= s.N) return;
  for (int k = threadIdx.x; k < n_sh; k += blockDim.x) sh[k] = 0.;
  __syncthreads();
  int cur = info_rep(s.info[b0]);
  int pos = b0;
  while (pos < b1) {
    // [pos, seg_end): slots of replica `cur` inside this block's chunk
    int seg_end = b1;
    if (info_rep(s.info[b1 - 1]) != cur) {
      int lo = pos, hi = b1 - 1;  // last slot with replica == cur
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (info_rep(s.info[mid]) == cur) lo = mid; else hi = mid - 1;
      }
      seg_end = lo + 1;
    }
    const RepDesc& R = s.reps[cur];
    for (int i = pos + threadIdx.x; i < seg_end; i += blockDim.x) {
      const int w = s.info[i];
      const int sp = info_species(w);
      if (!info_mobile(w) || sp == 3) continue;
      int zi = (int)(s.rz[i] * R.hist_inv_dz) + 1;
      zi = min(max(zi, 1), H) - 1;
      double* h = sh + (zi * 3 + sp) * 7;
      const double vx = s.vx[i], vy = s.vy[i], vz = s.vz[i];
      atomicAdd(h + 0, 1.);
      atomicAdd(h + 1, vx);
      atomicAdd(h + 2, vy);
      atomicAdd(h + 3, vz);
      atomicAdd(h + 4, vx * vx);
      atomicAdd(h + 5, vy * vy);
      atomicAdd(h + 6, vz * vz);
    }
    __syncthreads();
    double* g = prof + (size_t)cur * n_sh;
    for (int k = threadIdx.x; k < n_sh; k += blockDim.x) {
      double v = sh[k];
      if (v != 0.) atomicAdd(g + k, v);
      sh[k] = 0.;
    }
    __syncthreads();
    pos = seg_end;
    if (pos < b1) cur = info_rep(s.info[pos]);
  }
}

void launch_profiles(const DevState& s, const SimConst& C, cudaStream_t st, double* prof, int H) {
  // small chunks: enough blocks to fill the GPU for one large replica as for many small ones (a
  // block of sorted particles touches few bins, so its flush is short)
  const int chunk = 1024;
  const int g = (s.N + chunk - 1) / chunk;
  const size_t shm = sizeof(double) * H * 3 * 7;
  static size_t shm_set = 48 * 1024;
  if (shm > shm_set) {  // above 48 KB dynamic shared memory needs an explicit opt-in
    cudaFuncSetAttribute(k_profiles, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
    shm_set = shm;
  }
  k_profiles<<<g, 256, shm, st>>>(s, C, prof, H, chunk);
}

// energy record: out[k*nrep + r] = acc, acc = 0
__global__ void k_record(Acc acc, double* out) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  int n = NOBS * acc.nrep;
  if (k >= n) return;
  out[k] = acc.a[k];
  acc.a[k] = 0.;
}

// Observation quantities (observation.f90): one block per replica.  Rg^2 of each chain from its
// bonded beads unfolded one bond at a time (a coordinate that jumps by more than half the box
// from the previous bead is moved by one box length, observation.f90:187-201, all three axes as
// there), about the chain's centre of mass; averaged over the brush chains and over the melt
// chains (taken from the first melt particle on; the reference's melt loop starts at chain index
// n_chain with the melt stride, observation.f90:262, which only agrees when n_mon_d = n_mon).
// Momentum: sum of m v over the mobile particles.  Partial sums per thread, then a fixed-order
// tree: the result does not depend on timing.
constexpr int OBS_THREADS = 128;

__global__ void __launch_bounds__(OBS_THREADS) k_observe(DevState s, SimConst C, double* out) {
  __shared__ double part[OBS_THREADS][9];
  const int r = blockIdx.x;
  const RepDesc& R = s.reps[r];
  double acc[9] = {0., 0., 0., 0., 0., 0., 0., 0., 0.};
  const int nb = R.n_chain, nm = (R.n_mon_d > 0) ? R.n_chain_d : 0;
  const double half[3] = {0.5 * R.L[0], 0.5 * R.L[1], 0.5 * R.L[2]};
  for (int c = threadIdx.x; c < nb + nm; c += OBS_THREADS) {
    const bool brush = c < nb;
    const int len = brush ? R.n_mon : R.n_mon_d;
    const int t0 = R.p0 + (brush ? c * R.n_mon : R.part_init_d + (c - nb) * R.n_mon_d);
    double cm[3] = {0., 0., 0.}, rg[3] = {0., 0., 0.};
    for (int pass = 0; pass < 2; ++pass) {
      double prev[3] = {0., 0., 0.};
      for (int b = 0; b < len; ++b) {
        const int slot = s.slot_of_tag[t0 + b];
        double p[3] = {s.rx[slot], s.ry[slot], s.rz[slot]};
        if (b > 0) {
          for (int d = 0; d < 3; ++d) {
            if (p[d] - prev[d] > half[d]) p[d] -= R.L[d];
            else if (prev[d] - p[d] > half[d]) p[d] += R.L[d];
          }
        }
        for (int d = 0; d < 3; ++d) {
          prev[d] = p[d];
          if (pass == 0) cm[d] += p[d];
          else rg[d] += (p[d] - cm[d]) * (p[d] - cm[d]);
        }
      }
      if (pass == 0)
        for (int d = 0; d < 3; ++d) cm[d] /= (double)len;
    }
    for (int d = 0; d < 3; ++d) acc[(brush ? 0 : 3) + d] += rg[d] / (double)len;
  }
  for (int t = threadIdx.x; t < R.n_mon_tot; t += OBS_THREADS) {
    const int slot = s.slot_of_tag[R.p0 + t];
    const double m = C.mass[info_type(s.info[slot])];
    acc[6] += m * s.vx[slot];
    acc[7] += m * s.vy[slot];
    acc[8] += m * s.vz[slot];
  }
  for (int k = 0; k < 9; ++k) part[threadIdx.x][k] = acc[k];
  __syncthreads();
  for (int w = OBS_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < 9; ++k) part[threadIdx.x][k] += part[threadIdx.x + w][k];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    for (int d = 0; d < 3; ++d) {
      out[9 * r + d] = nb > 0 ? part[0][d] / (double)nb : 0.;
      out[9 * r + 3 + d] = nm > 0 ? part[0][3 + d] / (double)nm : 0.;
      out[9 * r + 6 + d] = part[0][6 + d];
    }
  }
}

__global__ void k_obs_accum(const double* __restrict__ rec, int nrep, const RepDesc* __restrict__ reps, SimConst C,
                            const double* __restrict__ obs, double* __restrict__ avg) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrep) return;
  mfa_energies e;
  record_energies(rec, nrep, r, reps[r], C, &e);
  mfa_virial w;
  record_virial(rec, nrep, r, reps[r], C, &w);
  double* a = avg + (size_t)r * NAVG;
  // observation.f90:140-170 (t_total = t_fluid: the wall beads do not move)
  const double vt = e.v_total, tt = e.t_fluid, et = e.e_total;
  const double vf = e.v_fluid_fluid + e.v_intra_molec + e.v_fluid_wall, tf = e.t_fluid, ef = e.v_fluid_fluid + e.t_fluid;
  a[A_COUNT] += 1.;
  a[A_VT] += vt; a[A_TT] += tt; a[A_ET] += et;
  a[A_VT2] += vt * vt; a[A_TT2] += tt * tt; a[A_ET2] += et * et;
  a[A_VF] += vf; a[A_TF] += tf; a[A_EF] += ef;
  a[A_VF2] += vf * vf; a[A_TF2] += tf * tf; a[A_EF2] += ef * ef;
  // observation.f90:247-291: Rg^2 means (brush, melt, their average), r_par_per2, momentum
  const double* o = obs + 9 * (size_t)r;
  for (int d = 0; d < 3; ++d) {
    a[A_MOM + d] += o[6 + d];
    a[A_RGB + d] += o[d];
    a[A_RGM + d] += o[3 + d];
    a[A_RGA + d] += 0.5 * (o[d] + o[3 + d]);
  }
  const double sb = o[0] + o[1] + o[2], sm = o[3] + o[4] + o[5];
  if (sb > 0.) a[A_RPP] += (o[2] - 0.5 * (o[0] + o[1])) / sb;  // (the reference divides by zero
  if (sm > 0.) a[A_RPP + 1] += (o[5] - 0.5 * (o[3] + o[4])) / sm;  //  when there are no chains)
  // obser_out.f90:309: press_tensor_mean
  for (int c = 0; c < 9; ++c) a[A_P + c] += w.pressure[c];
  // obser_out.f90:160-176: f_on_heads summed over the observations
  for (int c = 0; c < 6; ++c) a[A_FH + c] += rec[(size_t)(O_FH + c) * nrep + r];
}

void launch_obs_accum(const DevState& s, const SimConst& C, cudaStream_t st, const double* rec, const double* obs,
                      double* avg) {
  k_obs_accum<<<(s.nrep + 127) / 128, 128, 0, st>>>(rec, s.nrep, s.reps, C, obs, avg);
}

// The energy slots of the record (every slot before the virial) into the series ring at the
// current head; the head moves on in a separate one-thread kernel, after every thread has read it.
__global__ void k_series_store(const double* __restrict__ rec, int nrep, double* __restrict__ series,
                               long long* __restrict__ series_step, const long long* head, int cap,
                               const long long* steps_done) {
  const int slot = (int)(*head % cap);
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < O_VIR * nrep) series[(size_t)slot * O_VIR * nrep + k] = rec[k];
  if (k == 0) series_step[slot] = *steps_done;
}

__global__ void k_series_advance(long long* head) { *head += 1; }

void launch_series(const DevState& s, cudaStream_t st, const double* rec, double* series, long long* series_step,
                   long long* head, int cap) {
  const int n = O_VIR * s.nrep;
  k_series_store<<<(n + 255) / 256, 256, 0, st>>>(rec, s.nrep, series, series_step, head, cap, s.steps_done);
  k_series_advance<<<1, 1, 0, st>>>(head);
}

void launch_observe(const DevState& s, const SimConst& C, cudaStream_t st, double* out) {
  k_observe<<<s.nrep, OBS_THREADS, 0, st>>>(s, C, out);
}

void launch_record(Acc acc, double* out, cudaStream_t st) {
  int n = NOBS * acc.nrep;
  k_record<<<(n + 255) / 256, 256, 0, st>>>(acc, out);
}

// ---------------------------------------------------------------------------------------------
// Host layout <-> slot order
// ---------------------------------------------------------------------------------------------
__global__ void k_scatter(DevState s, const double* __restrict__ r, const double* __restrict__ v,
                          const double* __restrict__ a) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= s.N) return;
  int i = s.slot_of_tag[t];
  if (r) { s.rx[i] = r[3 * (size_t)t]; s.ry[i] = r[3 * (size_t)t + 1]; s.rz[i] = r[3 * (size_t)t + 2]; }
  if (v) { s.vx[i] = v[3 * (size_t)t]; s.vy[i] = v[3 * (size_t)t + 1]; s.vz[i] = v[3 * (size_t)t + 2]; }
  if (a) { s.ax[i] = a[3 * (size_t)t]; s.ay[i] = a[3 * (size_t)t + 1]; s.az[i] = a[3 * (size_t)t + 2]; }
}

void launch_scatter_state(const DevState& s, cudaStream_t st, const double* r, const double* v, const double* a) {
  k_scatter<<<(s.N + 255) / 256, 256, 0, st>>>(s, r, v, a);
}

__global__ void k_gather(DevState s, double* __restrict__ r, double* __restrict__ v, double* __restrict__ a,
                         double* __restrict__ f) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= s.N) return;
  int i = s.slot_of_tag[t];
  size_t o = 3 * (size_t)t;
  if (r) { r[o] = s.rx[i]; r[o + 1] = s.ry[i]; r[o + 2] = s.rz[i]; }
  if (v) { v[o] = s.vx[i]; v[o + 1] = s.vy[i]; v[o + 2] = s.vz[i]; }
  if (a) { a[o] = s.ax[i]; a[o + 1] = s.ay[i]; a[o + 2] = s.az[i]; }
  if (f) { f[o] = s.fx[i]; f[o + 1] = s.fy[i]; f[o + 2] = s.fz[i]; }
}

void launch_gather_state(const DevState& s, cudaStream_t st, double* r, double* v, double* a, double* f) {
  k_gather<<<(s.N + 255) / 256, 256, 0, st>>>(s, r, v, a, f);
}

__global__ void k_init_views(DevState s) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.N) return;
  int w = s.info[i];
  const RepDesc& R = s.reps[info_rep(w)];
  int4 q;
  store_views(s, i, R, s.rx[i], s.ry[i], s.rz[i], s.vx[i], s.vy[i], s.vz[i], w, s.tag[i], q);
  q.w = 0;
  s.ref[i] = q;
}

void launch_init_views(const DevState& s, cudaStream_t st) {
  k_init_views<<<(s.N + 255) / 256, 256, 0, st>>>(s);
}

// After a host update of the state (mfa_set_state): the views from the new r, v, and the skin
// test against the positions of the last rebuild, so that the lists are rebuilt only when some
// particle now sits more than skin/2 from where the lists were made.
__global__ void k_refresh_views(DevState s, float skin_half2) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.N) return;
  int w = s.info[i];
  const RepDesc& R = s.reps[info_rep(w)];
  int4 q;
  store_views(s, i, R, s.rx[i], s.ry[i], s.rz[i], s.vx[i], s.vy[i], s.vz[i], w, s.tag[i], q);
  const int4 q0 = s.ref[i];
  const float dx = i2f_fast(fx_diff(q.x, q0.x)) * R.ufx_f[0];
  const float dy = i2f_fast(fx_diff(q.y, q0.y)) * R.ufx_f[1];
  const float dz = i2f_fast(fx_diff(q.z, q0.z)) * R.ufx_f[2];
  if (info_mobile(w) && dx * dx + dy * dy + dz * dz > skin_half2) flag_rebuild(s, info_rep(w));
}

void launch_refresh_views(const DevState& s, const SimConst& C, cudaStream_t st) {
  k_refresh_views<<<(s.N + 255) / 256, 256, 0, st>>>(s, C.skin_half2_f);
}

}  // namespace mfa
