// mfa_obs.cuh -- energies, virial and pressure of one replica from an accumulator record, shared by
// the host (mfa_get_energies, mfa_get_virial) and the device (the observation averages), so both
// compose them the same way (verlet_velocities.f90:155-178, viscosity.f90:20-33).
#pragma once
#include <cstring>

#include "../../include/mfa_gpu.h"
#include "mfa_state.cuh"

namespace mfa {

// rec: slot-major [NOBS][nrep] record
__host__ __device__ inline void record_energies(const double* rec, int nrep, int rep, const RepDesc& R,
                                                const SimConst& C, mfa_energies* e) {
  auto A = [&](int slot) { return rec[(size_t)slot * nrep + rep]; };
  e->step = 0;
  e->v_fluid_fluid = A(O_VFF) + R.v_ffw;
  e->v_fluid_wall = A(O_VFW);
  e->v_wall_wall = R.v_ww;
  e->v_intra_molec = A(O_VINTRA);
  e->v_bend = A(O_VBEND);
  e->v_bend_melt = A(O_VBENDM);
  e->v_or = A(O_VOR);
  e->v_coul = C.charged ? A(O_VCOUL) + R.v_cself + A(O_VCOULK) + A(O_VDIP) : 0.;
  e->t_fluid = A(O_TFLUID);
  e->v_total = e->v_wall_wall + e->v_fluid_wall + e->v_fluid_fluid + e->v_intra_molec;
  if (C.bending) e->v_total += e->v_bend;
  if (C.orientation) e->v_total += e->v_or;
  if (C.bending_melt) e->v_total += e->v_bend_melt;
  if (C.charged) e->v_total += e->v_coul;
  e->e_total = e->v_total + e->t_fluid;  // t_total = t_fluid: the wall beads do not move
  e->inv_n = R.inv_n;
}

// The symmetric groups hold xx yy zz xy xz yz and are mirrored; the orientation group is a full
// tensor; the slab-dipole group follows from its energy u: diag(u, u, -u).
__host__ __device__ inline void record_virial(const double* rec, int nrep, int rep, const RepDesc& R,
                                              const SimConst& C, mfa_virial* o) {
  auto A = [&](int slot) { return rec[(size_t)slot * nrep + rep]; };
  double* grp[NVIR] = {o->pair, o->fene, o->bend, o->bend_melt, o->orientation, o->wall, o->kspace, o->dipole};
  o->step = 0;
  for (int g = 0; g < NVIR; ++g) {
    double* w = grp[g];
    for (int c = 0; c < 9; ++c) w[c] = A(O_VIR + 9 * g + c);
    if (g != V_OR)
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < a; ++b) w[3 * a + b] = w[3 * b + a];
  }
  const double ud = C.charged ? A(O_VDIP) : 0.;
  for (int c = 0; c < 9; ++c) o->dipole[c] = 0.;
  o->dipole[0] = o->dipole[4] = ud;
  o->dipole[8] = -ud;
  for (int c = 0; c < 9; ++c) o->kinetic[c] = A(O_KIN + c);
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < a; ++b) o->kinetic[3 * a + b] = o->kinetic[3 * b + a];
  o->volume = R.L[0] * R.L[1] * R.L[2];
  for (int c = 0; c < 9; ++c) {
    o->total[c] = 0.;
    for (int g = 0; g < NVIR; ++g) o->total[c] += grp[g][c];
    o->pressure[c] = (o->kinetic[c] + o->total[c]) / o->volume;
  }
}

// Observation averages per replica (observation.f90:17-301): slots of the accumulator
enum AvgSlot { A_COUNT = 0, A_VT, A_TT, A_ET, A_VT2, A_TT2, A_ET2, A_VF, A_TF, A_EF, A_VF2, A_TF2, A_EF2,
               A_MOM = 13, A_RGB = 16, A_RGM = 19, A_RGA = 22, A_RPP = 25, A_P = 27, A_FH = 36, NAVG = 42 };


}  // namespace mfa
