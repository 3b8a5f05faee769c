// mfa_integ.cuh -- the per-particle update of the mixed-precision integrator, shared by the
// integrator kernels (mfa_integrate.cu) and by the pair kernel that fuses the update of a step
// into its tail (mfa_forces.cu), so that both give the same bits.
#pragma once
#include "mfa_state.cuh"

namespace mfa {

// x -> wrapped x of verlet_positions.f90:170-186 (`> L` then `< 0`), decided on the bit pattern:
// for positive doubles integer order equals numeric order, so no FP64 compare is issued.
// The shift is chosen by integer selects, so one FP64 add is issued, not one per direction.
__device__ __forceinline__ double wrap_bits(double x, double L, long long Lbits) {
  const long long b = __double_as_longlong(x);
  const long long lb = __double_as_longlong(L), nlb = lb ^ (long long)0x8000000000000000ull;
  const long long ob = (b < 0 && b != (long long)0x8000000000000000ull) ? lb : (b > Lbits ? nlb : 0ll);
  return x + __longlong_as_double(ob);  // x + 0 keeps x (and -0.0 + 0 = +0, a zero all the same)
}

// The update of one mobile particle i (info word w) in the mixed path, after its force (Fx, Fy, Fz)
// for MODE >= 1; the views go to (pfx_out, vf_out).  Shared by k_int_mixed and by the pair kernel
// that fuses MODE 2 into its tail, so both give the same bits.
// verlet_positions.f90:214-247 (WALL 1 with a wall velocity): the sites of the first half of a
// replica's wall beads move by +va_spring_twall dt per step and the other half by
// -va_spring_twall dt, wrapped into [0, L) in x and y, and the beads sit on their sites.  Their
// velocity stays 0 (the reference assigns the wall beads none).  Writes the FP64 position
// (x, y, z out), returns the fixed-point view (w in .w) and raises the replica's rebuild flag
// when the bead has moved half the skin since the last rebuild (the test rounded as the mobile
// particles' test of the mixed path rounds it).  Shared by every position update, so all paths
// move a wall bead by the same bits.
__device__ __forceinline__ int4 move_wall_bead(const DevState& s, const SimConst& C, int i, int w, double& x,
                                               double& y, double& z) {
  const int rep = info_rep(w);
  const RepDesc& R = s.reps[rep];
  const bool first = s.tag[i] - R.p0 - R.n_mon_tot < (R.n_part - R.n_mon_tot) / 2;
  // rounded as written (no contraction into an FMA): the oracle's additions, bit for bit
  const double ddx = __dmul_rn(C.va_wall[0], C.dt), ddy = __dmul_rn(C.va_wall[1], C.dt);
  x = s.rx[i];
  y = s.ry[i];
  z = s.rz[i];
  x = first ? __dadd_rn(x, ddx) : __dsub_rn(x, ddx);
  y = first ? __dadd_rn(y, ddy) : __dsub_rn(y, ddy);
  if (x > R.L[0]) x -= R.L[0]; else if (x < 0.) x += R.L[0];
  if (y > R.L[1]) y -= R.L[1]; else if (y < 0.) y += R.L[1];
  s.rx[i] = x;
  s.ry[i] = y;
  int4 q;
  q.x = to_fx_periodic(x, R.sfx[0]);
  q.y = to_fx_periodic(y, R.sfx[1]);
  q.z = to_fx_z(z, R.sfx[2]);
  q.w = w;
  const int4 q0 = s.ref[i];
  const float dx = i2f_fast(fx_diff(q.x, q0.x)) * R.ufx_f[0];
  const float dy = i2f_fast(fx_diff(q.y, q0.y)) * R.ufx_f[1];
  const float dz = i2f_fast(fx_diff(q.z, q0.z)) * R.ufx_f[2];
  if (__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx))) > C.skin_half2_f) flag_rebuild(s, rep);
  return q;
}

template <int MODE, bool EFLAG>
__device__ __forceinline__ void int_mixed_particle(const DevState& s, const SimConst& C, int i, int w, float Fx,
                                                   float Fy, float Fz, int4* __restrict__ pfx_out,
                                                   float4* __restrict__ vf_out, float& ke, float* kin, float* fh) {
  const int rep = info_rep(w);
  {
    const RepDesc& R = s.reps[rep];
    const int t = info_type(w);
    double x = s.rx[i], y = s.ry[i], z = s.rz[i];
    double vx = s.vx[i], vy = s.vy[i], vz = s.vz[i];
    float ax, ay, az;
    if (MODE >= 1) {
      const float im = C.inv_mass_f[t];
      ax = Fx * im; ay = Fy * im; az = Fz * im;
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
        ax = ay = az = 0.f;
        Fx = Fy = Fz = 0.f;
      }
    } else {
      ax = d2f_fast(s.ax[i]); ay = d2f_fast(s.ay[i]); az = d2f_fast(s.az[i]);
    }
    const float h = (MODE == 2) ? C.dt_f : 0.5f * C.dt_f;
    const float dvx = h * ax, dvy = h * ay, dvz = h * az;
    if (EFLAG && MODE >= 1) {
      const float c = (MODE == 2) ? 0.5f : 1.0f;  // v(n) = v + dv/2 (MODE 2) or v + dv (MODE 1)
      const float ux = d2f_fast(vx) + c * dvx, uy = d2f_fast(vy) + c * dvy, uz = d2f_fast(vz) + c * dvz;
      ke = 0.5f * C.mass_f[t] * (ux * ux + uy * uy + uz * uz);
      sym_add(kin, C.mass_f[t], ux, uy, uz);
    }
    vx += f2d_fast(dvx);
    vy += f2d_fast(dvy);
    vz += f2d_fast(dvz);
    s.vx[i] = vx; s.vy[i] = vy; s.vz[i] = vz;
    if (MODE == 1) {
      s.ax[i] = f2d_fast(ax); s.ay[i] = f2d_fast(ay); s.az[i] = f2d_fast(az);
      s.fx[i] = f2d_fast(Fx); s.fy[i] = f2d_fast(Fy); s.fz[i] = f2d_fast(Fz);
    } else {
      x = wrap_bits(fma(C.dt, vx, x), R.L[0], R.Lbits[0]);
      y = wrap_bits(fma(C.dt, vy, y), R.L[1], R.Lbits[1]);
      z = fma(C.dt, vz, z);
      s.rx[i] = x; s.ry[i] = y; s.rz[i] = z;
      int4 q;
      q.x = to_fx_periodic(x, R.sfx[0]);
      q.y = to_fx_periodic(y, R.sfx[1]);
      q.z = to_fx_z(z, R.sfx[2]);
      q.w = w;
      pfx_out[i] = q;
      vf_out[i] = make_float4(d2f_fast(vx), d2f_fast(vy), d2f_fast(vz), __int_as_float(s.tag[i]));
      const int4 q0 = s.ref[i];
      const float dx = i2f_fast(fx_diff(q.x, q0.x)) * R.ufx_f[0];
      const float dy = i2f_fast(fx_diff(q.y, q0.y)) * R.ufx_f[1];
      const float dz = i2f_fast(fx_diff(q.z, q0.z)) * R.ufx_f[2];
      // rounded unmerged, so that the decision is the same in every kernel that makes it
      if (__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx))) > C.skin_half2_f) flag_rebuild(s, rep);
      const long long bx = __double_as_longlong(x), bz = __double_as_longlong(z);
      if (((bx >> 52) & 0x7FF) == 0x7FF || ((bz >> 52) & 0x7FF) == 0x7FF) atomicOr(s.status, ST_NAN);
    }
  }
}

}  // namespace mfa
