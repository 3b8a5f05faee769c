/*
 * mfa_oracle.c -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
 *
 * CPU FP64 restatement of mfa_brush's per-timestep MD-DPD hot path, written from the Fortran
 * sources of the reference (file:line cited per routine).  The reference itself cannot be built
 * here (no Fortran compiler; see the project design notes), so this restatement is the oracle.
 * It is pinned by the reference's own known-answer values in try/log (cut-off and shift tables,
 * the total LJ energy of try/conf_old, the first centre-of-mass velocity) and by analytic checks
 * (finite differences, Newton's third law, O(N^2) vs cell list).
 *
 * Deliberate differences from the Fortran, each behind a switch or documented:
 *   - DPD noise: the reference draws g ~ N(0,1) from a serial or wall-clock-seeded ziggurat
 *     (dpd_forces.f90:29-33), which cannot be reproduced.  Here g is a Box-Muller normal from a
 *     Philox2x32-10 stream keyed on (replica seed, step, min(tag), max(tag)), the same stream the
 *     CUDA product uses, so DPD-on parity is deterministic against this oracle.
 *   - Cell index clamping: get_cell (cell_list.f90:186-213) indexes out of range for a particle
 *     exactly on the upper box face or outside the channel; here the per-axis index is clamped.
 *   - DPD with its own cut-off reuses a stale 1/r in the reference for pairs outside the LJ
 *     range (fluid_fluid.f90:217-258 calls dpd_forces with inv_sqrt_r_2 from the last LJ pair);
 *     here 1/r of the current pair is used.
 *   - Explicit walls (WALL 1): wall beads are in the cell list, as in the BIN_TYPE 0 Verlet list
 *     (binning.f90:25,56); under BIN_TYPE 2 the reference lists mobile particles only and its
 *     wall beads would not interact at all.
 *   - Reference defects with a compat bit (MFA_COMPAT_*): 1/pi for 1/sqrt(pi) in ewald_real,
 *     force on i only, Coulomb only inside the LJ cut-off.
 *
 * Build: oracle/Makefile -> oracle/libmfa_oracle.so (gcc -O2 -fopenmp, plain C11).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/mfa_gpu.h"

#define MX MFA_MAX_TYPES
#define IDX(i, j) ((i) * MX + (j))

/* mfa_common.f90:315: pi is a default-REAL literal promoted to REAL(8). */
static double ref_pi(void) { return (double)3.1415926536f; }

/* Fortran x**n with an integer exponent: repeated multiplication. */
static inline double ipow(double x, int n) {
  double r = x;
  for (int k = 1; k < n; ++k) r *= x;
  return r;
}

/* ------------------------------------------------------------------------------------------
 * Philox2x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and a Box-Muller normal.
 * ---------------------------------------------------------------------------------------- */
static void philox2x32_10(uint32_t c[2], uint32_t k) {
  const uint32_t M = 0xD256D193u, W = 0x9E3779B9u;
  for (int r = 0; r < 10; ++r) {
    if (r > 0) k += W;
    uint64_t p = (uint64_t)M * c[0];
    uint32_t hi = (uint32_t)(p >> 32), lo = (uint32_t)p;
    c[0] = hi ^ k ^ c[1];
    c[1] = lo;
  }
}

/* Key of (replica seed, step): the low 32 bits of the step XOR the low half of the MurmurHash3
 * 64-bit finalizer of the seed. */
uint32_t orc_pair_key(uint64_t seed, int64_t step) {
  uint64_t h = seed;
  h ^= h >> 33;
  h *= 0xff51afd7ed558ccdULL;
  h ^= h >> 33;
  h *= 0xc4ceb9fe1a85ec53ULL;
  h ^= h >> 33;
  return (uint32_t)h ^ (uint32_t)(uint64_t)step;
}

/* Unit normal for the unordered pair (ta, tb) at `step`: counter (min tag, max tag), key
 * orc_pair_key(seed, step).  u1 in (0,1) and u2 in [0,1) are exact multiples of 2^-23 so FP32
 * and FP64 consumers see the same uniforms. */
double orc_pair_gauss(uint64_t seed, int64_t step, int32_t ta, int32_t tb) {
  uint32_t c[2] = {(uint32_t)(ta < tb ? ta : tb), (uint32_t)(ta < tb ? tb : ta)};
  philox2x32_10(c, orc_pair_key(seed, step));
  double u1 = ((double)(c[0] >> 9) + 0.5) * (1.0 / 8388608.0);
  double u2 = (double)(c[1] >> 9) * (1.0 / 8388608.0);
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

/* The raw block: counter (c0, c1), key k. */
void orc_philox2x32(uint32_t c0, uint32_t c1, uint32_t k, uint32_t* out2) {
  uint32_t c[2] = {c0, c1};
  philox2x32_10(c, k);
  memcpy(out2, c, 8);
}

/* ------------------------------------------------------------------------------------------
 * Derived tables: init_params.f90:393-887, init_config.f90:11-22, init_system.f90:172-187.
 * ---------------------------------------------------------------------------------------- */
int orc_derive_params(const mfa_inputs* in, mfa_params* p, mfa_system* s) {
  const mfa_flags* f = &in->flags;
  memset(p, 0, sizeof(*p));
  memset(s, 0, sizeof(*s));
  p->flags = *f;
  int nt = (f->wall == 1 && f->particle_4) ? 5 : 4; /* mfa_common.f90:46-60 */
  p->n_type = nt;
  int n = nt - 1; /* 0-based index of type n_type */
  const double c6 = (double)powf(2.0f, 1.0f / 6.0f); /* 2.**(1./6.) in single precision */
  const double c22 = (double)2.2f;
  double sigma[MX * MX], eps[MX * MX], range2[MX * MX];
  memset(sigma, 0, sizeof sigma);
  memcpy(eps, in->epsil, sizeof eps);
  double mass[MX], fric[MX];
  memcpy(mass, in->mass_type, sizeof mass);
  memcpy(fric, in->friction, sizeof fric);
  for (int i = 0; i < nt; ++i) sigma[IDX(i, i)] = in->sigma_ii[i];
  if (f->wall == 1 && !f->particle_4) { /* init_params.f90:175-185 (read loop, j_type==n_type) */
    sigma[IDX(n, n)] = 1.0;
    mass[n] = 1.0;
    fric[n] = fric[n - 1];
  }
  for (int i = 0; i < nt - 1; ++i) /* init_params.f90:405-429: sum rule */
    for (int j = i + 1; j < nt; ++j) {
      sigma[IDX(i, j)] = (sigma[IDX(i, i)] + sigma[IDX(j, j)]) / 2;
      sigma[IDX(j, i)] = sigma[IDX(i, j)];
    }
  if (f->solvent == 0 || f->solvent == 1) {
    if (!f->particle_4 && f->wall != 1)
      for (int i = 0; i < nt; ++i) sigma[IDX(i, n)] = sigma[IDX(n, i)] = 0.0;
  } else { /* non-additive: init_params.f90:432-449 */
    sigma[IDX(1, 2)] = sigma[IDX(2, 1)] = sigma[IDX(0, 2)] = sigma[IDX(2, 0)] = in->delta_sig[0];
    if (f->particle_4) {
      sigma[IDX(1, 3)] = sigma[IDX(3, 1)] = sigma[IDX(0, 3)] = sigma[IDX(3, 0)] = in->delta_sig[1];
      sigma[IDX(2, 3)] = sigma[IDX(3, 2)] = in->delta_sig[2];
    }
  }
  for (int i = 0; i < nt; ++i) /* init_params.f90:465-470 */
    for (int j = 0; j < nt; ++j) {
      p->sigma[IDX(i, j)] = sigma[IDX(i, j)];
      p->sigma_2[IDX(i, j)] = sigma[IDX(i, j)] * sigma[IDX(i, j)];
      p->epsil[IDX(i, j)] = 4. * eps[IDX(i, j)];
    }
  if (f->wall != 1) p->epsil[IDX(0, 0)] = 0.; /* init_params.f90:491-493 */
  /* cut-offs: init_params.f90:497-725 */
#define SQ(x) ((x) * (x))
  for (int i = 0; i < nt; ++i)
    for (int j = 0; j < nt; ++j) range2[IDX(i, j)] = SQ(c6 * sigma[IDX(i, j)]);
  range2[IDX(0, n)] = SQ(c22 * sigma[IDX(0, n)]);
  range2[IDX(n, 0)] = SQ(c22 * sigma[IDX(n, 0)]);
  if (f->wall == 1) {
    if (f->solvent == 0 || f->solvent == 3) {
      for (int i = 0; i < nt; ++i)
        for (int j = 0; j < nt; ++j) range2[IDX(i, j)] = SQ(2. * c6 * sigma[IDX(1, 1)]);
      range2[IDX(0, n)] = range2[IDX(n, 0)] = range2[IDX(n, n)] = 0.;
    } else {
      for (int i = 0; i < nt - 1; ++i)
        for (int j = 0; j < nt - 1; ++j) range2[IDX(i, j)] = SQ(c6 * sigma[IDX(i, j)]);
    }
  } else { /* WALL 2/3/4 */
    if (f->solvent == 0) {
      for (int i = 0; i < nt; ++i)
        for (int j = 0; j < nt; ++j) range2[IDX(i, j)] = SQ(2. * c6 * sigma[IDX(i, j)]);
      if (!f->particle_4)
        for (int i = 0; i < nt; ++i) range2[IDX(i, n)] = range2[IDX(n, i)] = 0.;
    }
    if (f->solvent == 3)
      for (int i = 0; i < nt; ++i)
        for (int j = 0; j < nt; ++j) range2[IDX(i, j)] = SQ(2. * c6 * sigma[IDX(i, j)]);
    if (f->hydrophobia) {
      range2[IDX(0, 2)] = SQ(c6 * sigma[IDX(0, 2)]);
      range2[IDX(1, 2)] = SQ(c6 * sigma[IDX(1, 2)]);
      range2[IDX(2, 0)] = SQ(c6 * sigma[IDX(2, 0)]);
      range2[IDX(2, 1)] = SQ(c6 * sigma[IDX(2, 1)]);
    }
    if (f->brush_in_good_sv) {
      range2[IDX(0, 1)] = SQ(c6 * sigma[IDX(0, 1)]);
      range2[IDX(0, 0)] = SQ(c6 * sigma[IDX(0, 0)]);
      range2[IDX(1, 1)] = SQ(c6 * sigma[IDX(1, 1)]);
      range2[IDX(1, 0)] = SQ(c6 * sigma[IDX(1, 0)]);
    }
  }
  if (f->wall == 2) { /* init_params.f90:592-601 */
    for (int i = 0; i < nt; ++i) {
      p->sigma_wall[i] = (in->sigma_w + sigma[IDX(i, i)]) / 2;
      p->a_wall[i] = in->a_w;
    }
    if (f->particle_4) {
      p->sigma_wall[3] = (in->sigma_w4 + sigma[IDX(3, 3)]) / 2.;
      p->a_wall[3] = in->a_w4;
    }
  }
  if (!f->particle_4) {
    if (f->wall == 2)
      for (int i = 0; i < nt; ++i) range2[IDX(i, n)] = range2[IDX(n, i)] = 0.;
  } else {
    if (f->wall == 1) {
      if (f->solvent == 1)
        for (int i = 0; i < nt; ++i) range2[IDX(i, n)] = range2[IDX(n, i)] = SQ(c6 * sigma[IDX(i, n)]);
      if (f->solvent == 0)
        for (int i = 0; i < nt; ++i) range2[IDX(i, n)] = range2[IDX(n, i)] = SQ(c22 * sigma[IDX(i, n)]);
    }
    int i4 = in->inter4;
    if (i4 >= 1 && i4 <= 3) {
      for (int i = 0; i < 3; ++i) {
        range2[IDX(i, 3)] = SQ(c6 * sigma[IDX(i, 3)]);
        range2[IDX(3, i)] = SQ(c6 * sigma[IDX(3, i)]);
      }
      range2[IDX(3, 3)] = (i4 == 1) ? SQ(c6 * sigma[IDX(3, 3)]) : SQ(2. * (c6 * sigma[IDX(3, 3)]));
    } else if (i4 == 4) {
      for (int i = 0; i < 3; ++i) {
        range2[IDX(i, 3)] = SQ(2. * c6 * sigma[IDX(i, 3)]);
        range2[IDX(3, i)] = SQ(2. * c6 * sigma[IDX(3, i)]);
      }
      range2[IDX(3, 3)] = SQ(2. * (c6 * sigma[IDX(3, 3)]));
    }
  }
  if (f->system == 0 || f->system == 1 || f->system == 3) range2[IDX(0, 0)] = 0.; /* :716-719 */
  double rmax2 = 0.;
  for (int i = 0; i < nt; ++i)
    for (int j = 0; j < nt; ++j) {
      double r2 = range2[IDX(j, i)];
      p->range_2[IDX(j, i)] = r2;
      if (r2 > 0.0) {
        double r = ipow(sigma[IDX(j, i)] * sigma[IDX(j, i)] / r2, 3);
        p->e_shift[IDX(j, i)] = r * (r - 1.);
      } else {
        p->e_shift[IDX(j, i)] = 0.0;
      }
      p->inv_range_2[IDX(i, j)] = (r2 != 0) ? 1. / r2 : 0.;
      if (r2 > rmax2) rmax2 = r2;
    }
  p->r_cut_max = sqrt(rmax2);
  if (f->dpd_cut_off > 0) { /* init_params.f90:796-807: the macro is a single-precision literal */
    double rd = (double)(float)f->dpd_cut_off;
    if (rd > p->r_cut_max) p->r_cut_max = rd;
    p->r_cut_dpd_2 = rd * rd;
  }
  p->skin = (double)0.4f;
  p->dt = in->dt;
  p->temp = in->temp;
  for (int i = 0; i < nt; ++i) p->mass_type[i] = mass[i];
  p->friction1 = fric[0];
  p->sig = sqrt(2. * in->temp * fric[0] / in->dt); /* init_params.f90:887 */
  p->a_w = in->a_w;
  p->sigma_w = in->sigma_w;
  p->r_chain_2 = in->r_chain * in->r_chain; /* init_params.f90:393-396 */
  p->inv_r_chain_2 = 1. / p->r_chain_2;
  p->k_chain = in->k_chain * p->r_chain_2;
  p->k_bend = in->k_bend;
  p->alpha_eq = in->alpha_eq;
  p->k_or = in->k_bend; /* orientation.f90:14-15 */
  p->alpha_or = 0.;
  p->bend_form = in->bend_form;
  for (int d = 0; d < 3; ++d) p->const_force[d] = in->const_force[d];
  for (int i = 0; i < MX; ++i) p->charge[i] = in->charge[i];
  p->alpha_c = in->alpha_c;
  p->sqrt_alpha = sqrt(in->alpha_c); /* init_config.f90:231-232 */
  p->inv_sqrt_pi = (in->compat & MFA_COMPAT_EWALD_INV_PI) ? 1. / ref_pi() : 1. / sqrt(ref_pi());
  p->n_kmax = in->n_kmax;
  p->rc_coul_2 = in->rc_coul * in->rc_coul;
  p->compat = in->compat;
  p->hist_dim = in->hist_dim > 0 ? in->hist_dim : 200;
  /* heads sheared with the walls (verlet_velocities.f90:111-124); refused with the body force
     (init_params.f90:899-907) and, with explicit walls (whose sites move too), for a z velocity */
  if (in->va_spring_twall[0] != 0. || in->va_spring_twall[1] != 0. || in->va_spring_twall[2] != 0.) {
    if (f->poiseuille || (f->wall == 1 && in->va_spring_twall[2] != 0.)) return -2;
    p->va_wall[0] = in->va_spring_twall[0];
    p->va_wall[1] = in->va_spring_twall[1];
  }
  p->r_2_min_init = 0.;
  p->r_2_min_time = 0.;
  /* box and counts */
  s->boundary[0] = in->x_space * (double)in->n_cell_w_x;
  s->boundary[1] = in->y_space * (double)in->n_cell_w_y;
  s->boundary[2] = in->z_space_wall;
  s->n_mon = in->n_mon;
  s->n_chain = in->n_chain;
  s->n_mon_d = in->n_mon_d;
  s->n_chain_d = in->n_chain_d;
  s->n_mon_e = f->particle_4 ? in->n_mon_e : 0;
  s->n_chain_e = f->particle_4 ? in->n_chain_e : 0;
  s->n_mon_tot = in->n_mon * in->n_chain + in->n_mon_d * in->n_chain_d + s->n_mon_e * s->n_chain_e;
  s->n_part = s->n_mon_tot + (f->wall == 1 ? 4 * in->n_cell_w_x * in->n_cell_w_y : 0);
  s->s_time = in->s_time;
  s->seed = (uint64_t)in->iseed;
  return 0;
#undef SQ
}

/* init_force_switch_on.f90:12-21 */
void orc_force_switch_on(mfa_params* p, int64_t n_relax) {
  double maxsig = 0.;
  for (int i = 0; i < p->n_type; ++i)
    for (int j = 0; j < p->n_type; ++j)
      if (p->sigma[IDX(i, j)] > maxsig) maxsig = p->sigma[IDX(i, j)];
  p->r_2_min_init = ipow((double)0.9f * maxsig, 2);
  p->r_2_min_time = ((double)n_relax * p->dt < 40.) ? 40. : (double)n_relax * p->dt;
}

/* ------------------------------------------------------------------------------------------
 * System state
 * ---------------------------------------------------------------------------------------- */
typedef struct orc_sys {
  mfa_params p;
  mfa_system s;
  int n, nm;          /* n_part, n_mon_tot */
  int part_init_d, part_init_e;
  int32_t* a_type;    /* 1-based types */
  double *r0, *v, *a, *force, *mass, *inv_mass, *ext_force, *q;
  /* cell list (cell_list.f90) */
  int l_box, nc[3], nct, n_nei;
  double l_cell[3], inv_l_cell[3];
  int *part_in_cell, *r_nei, *l_nei, *cell_neigh_ls; /* 1-based particle ids, 0 = none */
  /* energies */
  double v_ff, v_coul, v_fw, v_ww, v_intra, v_bend, v_bend_melt, v_or, t_fluid;
  double f_heads[6];  /* -sum of the head forces, chains 1..n_chain/2 then the others */
  double r_2_min;
  int64_t step;       /* absolute step being computed: s_time + i_time - 1 */
  int i_time;
  /* ewald */
  int nk;
  double *kv, *k2, *ik2, inv_V_k, lz_half, v_coul_self, fac_alpha;
  /* profiles */
  int hist;
  double *dens, *vp, *vp2;
  int64_t n_obs;
  /* virial W_ab = minus the derivative of the energy under the strain r_a -> r_a + e r_b (box,
     walls and positions deformed together).  For the pair, bond, angle and wall terms that is the
     sum over the terms of F_a r_b (F on a particle, r its position relative to the other
     particles of the term, or to the wall plane); the k-space and slab-dipole energies depend on
     the volume as well.  Groups: 0 pair (LJ + DPD + real-space Coulomb), 1 FENE, 2 brush bending,
     3 melt bending, 4 orientation, 5 walls (zz), 6 k-space, 7 slab dipole; each routine sets its
     own group */
  double vir[8][9];
  /* per-particle force scale: the sum of the magnitudes of every force term acting on the
     particle (NULL unless enabled by orc_track_force_scale) */
  double* fscale;
} orc_sys;

static inline void fsc(const orc_sys* o, int i0, const double* f) {
  if (o->fscale) o->fscale[i0] += sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
}
static inline void fsc_mag(const orc_sys* o, int i0, double m) {
  if (o->fscale) o->fscale[i0] += fabs(m);
}
/* W_ab += f_a r_b */
static inline void vir_add(double* w, const double* f, const double* r) {
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) w[3 * a + b] += f[a] * r[b];
}

static int get_cell(const orc_sys* o, const double* r) {
  /* cell_list.f90:186-213 with per-axis clamping (see header) */
  int pc = 1, pf = 1;
  for (int d = 0; d < 3; ++d) {
    int c = (int)(r[d] * o->inv_l_cell[d]);
    if (c < 0) c = 0;
    if (c > o->nc[d] - 1) c = o->nc[d] - 1;
    pc += pf * c;
    pf *= o->nc[d];
  }
  return pc;
}

/* make_cell_list2, n_dim = 3, SYMMETRY 0 (cell_list.f90:337-403) */
static void make_cell_list2(int in_cell, const int* nc, int n_nei, int* out) {
  int z_cell = (in_cell - 1) / (nc[0] * nc[1]) + 1;
  int y_cell = (in_cell - nc[0] * nc[1] * (z_cell - 1) - 1) / nc[0] + 1;
  int x_cell = in_cell - nc[0] * nc[1] * (z_cell - 1) - nc[0] * (y_cell - 1);
  int il = 0;
  if (n_nei == 13) {
    for (int i = 2; i <= 3; ++i)
      for (int j = 1; j <= 3; ++j) {
        if (i == 2 && j <= 1) continue;
        for (int k = 1; k <= 3; ++k) {
          if (i == 2 && j == 2 && k >= 3) continue;
          int jc = in_cell + i - 2 + (j - 2) * nc[0] + (k - 2) * nc[1] * nc[0];
          if (jc == in_cell) continue;
          if (x_cell == 1 && i == 1) jc += nc[0];
          if (x_cell == nc[0] && i == 3) jc -= nc[0];
          if (y_cell == 1 && j == 1) jc += nc[0] * nc[1];
          if (y_cell == nc[1] && j == 3) jc -= nc[0] * nc[1];
          if (z_cell + k - 2 < 1) jc = 0;
          if (z_cell + k - 2 > nc[2]) jc = 0;
          out[il++] = jc;
        }
      }
  } else { /* 62 */
    for (int i = 2; i <= 4; ++i)
      for (int j = 0; j <= 4; ++j) {
        if (i == 2 && j <= 1) continue;
        for (int k = 0; k <= 4; ++k) {
          if (i == 2 && j == 2 && k >= 3) continue;
          int jc = in_cell + i - 2 + (j - 2) * nc[0] + (k - 2) * nc[1] * nc[0];
          if (jc == in_cell) continue;
          if (x_cell + i - 2 > nc[0]) jc -= nc[0];
          if (y_cell + j - 2 < 1) jc += nc[0] * nc[1];
          if (y_cell + j - 2 > nc[1]) jc -= nc[0] * nc[1];
          if (z_cell + k - 2 < 1) jc = 0;
          if (z_cell + k - 2 > nc[2]) jc = 0;
          out[il++] = jc;
        }
      }
  }
}

int orc_cell_neigh_list(const int32_t* n_cells, int32_t n_nei, int32_t* out) {
  int nc[3] = {n_cells[0], n_cells[1], n_cells[2]};
  int nct = nc[0] * nc[1] * nc[2];
  for (int c = 1; c <= nct; ++c) make_cell_list2(c, nc, n_nei, out + (size_t)(c - 1) * n_nei);
  return 0;
}

/* make_binning + neigh_list + get_cell_neigh_list (cell_list.f90:56-158,270-283). */
int orc_make_cell_list(orc_sys* o, int l_box) {
  o->l_box = l_box;
  double rc = o->p.r_cut_max;
  /* an own real-space Coulomb cut-off (not expressible in the reference) widens the cells */
  if ((o->p.flags.system == 2 || o->p.flags.system == 3) && o->p.rc_coul_2 > 0. &&
      !(o->p.compat & MFA_COMPAT_COUL_IN_LJ) && sqrt(o->p.rc_coul_2) > rc)
    rc = sqrt(o->p.rc_coul_2);
  for (int d = 0; d < 3; ++d) {
    o->nc[d] = (l_box == 1) ? (int)(o->s.boundary[d] / rc) : (int)(o->s.boundary[d] / (rc / 2.));
    if (o->nc[d] < 1) o->nc[d] = 1;
    o->l_cell[d] = o->s.boundary[d] / (double)(float)o->nc[d];
    o->inv_l_cell[d] = 1 / o->l_cell[d];
  }
  o->n_nei = (l_box == 1) ? 13 : 62;
  o->nct = o->nc[0] * o->nc[1] * o->nc[2];
  free(o->part_in_cell);
  free(o->cell_neigh_ls);
  o->part_in_cell = (int*)calloc((size_t)o->nct + 1, sizeof(int));
  o->cell_neigh_ls = (int*)malloc((size_t)o->nct * o->n_nei * sizeof(int));
  for (int i = 1; i <= o->n; ++i) o->r_nei[i] = o->l_nei[i] = 0;
  /* The linked-cell list covers the mobile particles only (init_config.f90:270), so under
     BIN_TYPE 2 explicit wall beads never interact.  With explicit walls (WALL 1) the list takes
     every particle, walls included, as the BIN_TYPE 0 Verlet list does (binning.f90:25,56). */
  const int n_listed = (o->p.flags.wall == 1) ? o->n : o->nm;
  for (int i = 1; i <= n_listed; ++i) {
    int pc = get_cell(o, &o->r0[3 * (i - 1)]);
    if (o->part_in_cell[pc] == 0) {
      o->part_in_cell[pc] = i;
    } else {
      int j = o->part_in_cell[pc];
      o->part_in_cell[pc] = i;
      o->r_nei[i] = j;
      o->l_nei[i] = 0;
      o->l_nei[j] = i;
    }
  }
  o->part_in_cell[0] = 0;
  orc_cell_neigh_list(o->nc, o->n_nei, o->cell_neigh_ls);
  return 0;
}

int orc_cell_info(orc_sys* o, int32_t* cell_of, int32_t* counts, int32_t* n_cells) {
  for (int i = 1; i <= o->nm; ++i) cell_of[i - 1] = get_cell(o, &o->r0[3 * (i - 1)]);
  if (counts) {
    for (int c = 0; c <= o->nct; ++c) {
      int k = 0;
      for (int j = o->part_in_cell[c]; j != 0; j = o->r_nei[j]) ++k;
      counts[c] = k;
    }
  }
  for (int d = 0; d < 3; ++d) n_cells[d] = o->nc[d];
  return o->nct;
}

/* update_part_cell (cell_list.f90:215-268) */
static void update_part_cell(orc_sys* o, int i, int old_cell) {
  int nc_ = get_cell(o, &o->r0[3 * (i - 1)]);
  if (nc_ == old_cell) return;
  if (o->part_in_cell[old_cell] == i) {
    int j = o->r_nei[i];
    o->part_in_cell[old_cell] = j;
    if (j != 0) o->l_nei[j] = 0;
  } else {
    int j = o->r_nei[i];
    o->r_nei[o->l_nei[i]] = j;
    if (j != 0) o->l_nei[j] = o->l_nei[i];
  }
  if (o->part_in_cell[nc_] == 0) {
    o->part_in_cell[nc_] = i;
    o->l_nei[i] = 0;
    o->r_nei[i] = 0;
  } else {
    int j = o->part_in_cell[nc_];
    o->part_in_cell[nc_] = i;
    o->r_nei[i] = j;
    o->l_nei[i] = 0;
    o->l_nei[j] = i;
  }
}

orc_sys* orc_create(const mfa_params* p, const mfa_system* s, const int32_t* a_type,
                    const double* r0, const double* v, const double* a) {
  orc_sys* o = (orc_sys*)calloc(1, sizeof(orc_sys));
  o->p = *p;
  o->s = *s;
  o->n = s->n_part;
  o->nm = s->n_mon_tot;
  o->part_init_d = s->n_mon * s->n_chain;
  o->part_init_e = o->part_init_d + s->n_mon_d * s->n_chain_d;
  size_t n3 = (size_t)3 * o->n;
  o->a_type = (int32_t*)malloc(sizeof(int32_t) * o->n);
  memcpy(o->a_type, a_type, sizeof(int32_t) * o->n);
  o->r0 = (double*)malloc(n3 * 8);
  o->v = (double*)malloc(n3 * 8);
  o->a = (double*)malloc(n3 * 8);
  o->force = (double*)calloc(n3, 8);
  o->ext_force = (double*)calloc(n3, 8);
  memcpy(o->r0, r0, n3 * 8);
  memcpy(o->v, v, n3 * 8);
  memcpy(o->a, a, n3 * 8);
  o->mass = (double*)malloc(8 * (size_t)o->n);
  o->inv_mass = (double*)malloc(8 * (size_t)o->n);
  o->q = (double*)calloc((size_t)o->n, 8);
  for (int i = 0; i < o->n; ++i) { /* init_config.f90:326-329 */
    o->mass[i] = p->mass_type[a_type[i] - 1];
    o->inv_mass[i] = 1. / p->mass_type[a_type[i] - 1];
  }
  for (int i = 0; i < o->nm; ++i) { /* init_config.f90:223-228, 370-378 */
    o->q[i] = (p->flags.system == 2 || p->flags.system == 3) ? p->charge[a_type[i] - 1] : 0.;
    if (p->flags.poiseuille && a_type[i] != 1)
      for (int d = 0; d < 3; ++d) o->ext_force[3 * i + d] = o->mass[i] * p->const_force[d];
  }
  o->r_nei = (int*)calloc((size_t)o->n + 1, sizeof(int));
  o->l_nei = (int*)calloc((size_t)o->n + 1, sizeof(int));
  o->step = s->s_time;
  o->i_time = 0;
  o->hist = p->hist_dim;
  o->dens = (double*)calloc((size_t)o->hist * 3, 8);
  o->vp = (double*)calloc((size_t)o->hist * 9, 8);
  o->vp2 = (double*)calloc((size_t)o->hist * 9, 8);
  o->lz_half = s->boundary[2] / 2.;
  if (p->flags.system == 2 || p->flags.system == 3) {
    double vs = 0.;
    for (int i = 0; i < o->nm; ++i) vs -= o->q[i] * o->q[i];
    o->v_coul_self = vs * p->sqrt_alpha / sqrt(ref_pi()); /* init_config.f90:237-241 */
  }
  orc_make_cell_list(o, p->flags.l_box > 0 ? p->flags.l_box : 1);
  return o;
}

void orc_destroy(orc_sys* o) {
  if (!o) return;
  free(o->a_type); free(o->r0); free(o->v); free(o->a); free(o->force); free(o->ext_force);
  free(o->mass); free(o->inv_mass); free(o->q); free(o->r_nei); free(o->l_nei);
  free(o->part_in_cell); free(o->cell_neigh_ls); free(o->kv); free(o->k2); free(o->ik2);
  free(o->dens); free(o->vp); free(o->vp2); free(o->fscale);
  free(o);
}

void orc_get_state(const orc_sys* o, double* r0, double* v, double* a, double* f) {
  size_t n3 = (size_t)3 * o->n * 8;
  if (r0) memcpy(r0, o->r0, n3);
  if (v) memcpy(v, o->v, n3);
  if (a) memcpy(a, o->a, n3);
  if (f) memcpy(f, o->force, n3);
}
void orc_set_state(orc_sys* o, const double* r0, const double* v, const double* a) {
  size_t n3 = (size_t)3 * o->n * 8;
  if (r0) memcpy(o->r0, r0, n3);
  if (v) memcpy(o->v, v, n3);
  if (a) memcpy(o->a, a, n3);
  orc_make_cell_list(o, o->l_box);
}
void orc_set_force(orc_sys* o, const double* f) { memcpy(o->force, f, (size_t)3 * o->n * 8); }
void orc_set_step(orc_sys* o, int64_t step) { o->step = step; }
int64_t orc_get_step(const orc_sys* o) { return o->step; }
void orc_set_r2min(orc_sys* o, double r2min) { o->r_2_min = r2min; }

/* Energies in mfa_energies field order (step excluded). */
/* Observation quantities (observation.f90:187-291): out[0..2] brush Rg^2 per axis (chains unfolded
 * one bond at a time, observation.f90:187-201, then about the centre of mass, 214-245), out[3..5]
 * the same for the melt chains counted from the first melt particle (the reference's loop at
 * observation.f90:262 starts at chain index n_chain with the melt stride, which agrees only when
 * n_mon_d = n_mon), out[6..8] the momentum (286-291), out[9..14] the head forces of the last
 * verlet_velocities. */
static void chain_rg2(const orc_sys* o, int t0, int len, double* rg) {
  const double* L = o->s.boundary;
  double cm[3] = {0, 0, 0}, prev[3] = {0, 0, 0};
  double* sp = (double*)malloc(sizeof(double) * 3 * (size_t)len);
  for (int b = 0; b < len; ++b) {
    for (int d = 0; d < 3; ++d) {
      double x = o->r0[3 * (t0 + b) + d];
      if (b > 0) {
        if (x - prev[d] > 0.5 * L[d]) x -= L[d];
        else if (prev[d] - x > 0.5 * L[d]) x += L[d];
      }
      prev[d] = x;
      sp[3 * b + d] = x;
      cm[d] += x;
    }
  }
  for (int d = 0; d < 3; ++d) cm[d] /= (double)len;
  for (int d = 0; d < 3; ++d) {
    double acc = 0.;
    for (int b = 0; b < len; ++b) acc += (sp[3 * b + d] - cm[d]) * (sp[3 * b + d] - cm[d]);
    rg[d] = acc / (double)len;
  }
  free(sp);
}

void orc_observe(const orc_sys* o, double* out) {
  for (int k = 0; k < 15; ++k) out[k] = 0.;
  const mfa_system* s = &o->s;
  double rg[3];
  for (int c = 0; c < s->n_chain; ++c) {
    chain_rg2(o, c * s->n_mon, s->n_mon, rg);
    for (int d = 0; d < 3; ++d) out[d] += rg[d];
  }
  if (s->n_chain > 0)
    for (int d = 0; d < 3; ++d) out[d] /= (double)s->n_chain;
  if (s->n_mon_d > 0 && s->n_chain_d > 0) {
    for (int c = 0; c < s->n_chain_d; ++c) {
      chain_rg2(o, o->part_init_d + c * s->n_mon_d, s->n_mon_d, rg);
      for (int d = 0; d < 3; ++d) out[3 + d] += rg[d];
    }
    for (int d = 0; d < 3; ++d) out[3 + d] /= (double)s->n_chain_d;
  }
  for (int i = 0; i < o->nm; ++i)
    for (int d = 0; d < 3; ++d) out[6 + d] += o->mass[i] * o->v[3 * i + d];
  for (int k = 0; k < 6; ++k) out[9 + k] = o->f_heads[k];
}

void orc_get_energies(const orc_sys* o, double* e) {
  e[0] = o->v_ff; e[1] = o->v_fw; e[2] = o->v_ww; e[3] = o->v_intra;
  e[4] = o->v_bend; e[5] = o->v_bend_melt; e[6] = o->v_or; e[7] = o->v_coul; e[8] = o->t_fluid;
}

void orc_zero_force(orc_sys* o) {
  memset(o->force, 0, (size_t)3 * o->n * 8);
  if (o->fscale) memset(o->fscale, 0, (size_t)o->n * 8);
  memset(o->vir, 0, sizeof o->vir);
}

/* Per-particle force scale (test aid: the conditioning of each particle's force sum). */
void orc_track_force_scale(orc_sys* o, int on) {
  free(o->fscale);
  o->fscale = on ? (double*)calloc((size_t)o->n, 8) : NULL;
}
void orc_get_force_scale(const orc_sys* o, double* out) {
  if (o->fscale) memcpy(out, o->fscale, (size_t)o->n * 8);
  else memset(out, 0, (size_t)o->n * 8);
}
/* out[9 g + 3 a + b] = W_ab of group g (8 groups, see orc_sys::vir) */
void orc_get_virial(const orc_sys* o, double* out) { memcpy(out, o->vir, sizeof o->vir); }
/* Kinetic tensor sum m v_a v_b over the mobile particles (viscosity.f90:20-27). */
void orc_kinetic_tensor(const orc_sys* o, double* out) {
  for (int k = 0; k < 9; ++k) out[k] = 0.;
  for (int i = 0; i < o->nm; ++i)
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) out[3 * a + b] += o->mass[i] * o->v[3 * i + a] * o->v[3 * i + b];
}

/* ------------------------------------------------------------------------------------------
 * Pair interaction of fluid_fluid.f90:97-261 / 276-436 for the ordered pair (i, j), 1-based.
 * fi accumulates the LJ force on i (f_ipart); force_tmp receives the DPD and Coulomb terms on
 * i and j, and the LJ reaction on j.  Returns nothing; energies via pointers.
 * ---------------------------------------------------------------------------------------- */
/* Force scale of a DPD pair (1-based i, j): the random and dissipative terms at unit weight,
 * sigma |g| and gamma (|v_i| + |v_j|).  The weight 1 - r/r_c is itself a difference of numbers of
 * order one, so the error of either term does not shrink with the weight. */
static inline void dpd_scale(const orc_sys* o, int i, int j, double g) {
  if (!o->fscale) return;
  const double* vi = &o->v[3 * (i - 1)];
  const double* vj = &o->v[3 * (j - 1)];
  const double m = o->p.sig * fabs(g) +
                   o->p.friction1 * (sqrt(vi[0] * vi[0] + vi[1] * vi[1] + vi[2] * vi[2]) +
                                     sqrt(vj[0] * vj[0] + vj[1] * vj[1] + vj[2] * vj[2]));
  o->fscale[i - 1] += m;
  o->fscale[j - 1] += m;
}

static inline void pair_ij(const orc_sys* o, int i, int j, double* fi, double* force_tmp,
                           double* v_ff, double* v_coul, double* w) {
  const mfa_params* p = &o->p;
  int ti = o->a_type[i - 1] - 1, tj = o->a_type[j - 1] - 1;
  double r_cut2 = p->range_2[IDX(ti, tj)];
  const double* ri = &o->r0[3 * (i - 1)];
  const double* rj = &o->r0[3 * (j - 1)];
  double dr[3] = {ri[0] - rj[0], ri[1] - rj[1], ri[2] - rj[2]};
  const double* L = o->s.boundary;
  dr[0] = dr[0] - L[0] * (double)(int64_t)(2. * dr[0] * (1. / L[0]));
  dr[1] = dr[1] - L[1] * (double)(int64_t)(2. * dr[1] * (1. / L[1]));
  double r_2 = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
  double r_2_raw = r_2;
  double inv_sqrt_r_2 = 0.;
  int in_lj = r_2 < r_cut2;
  int dpd = (p->flags.thermostat == 0);
  if (in_lj) {
    if (p->flags.force_switch_on && r_2 < o->r_2_min) r_2 = o->r_2_min;
    double inv_r_2 = 1. / r_2;
    inv_sqrt_r_2 = sqrt(1. / r_2);
    double l_eps = p->epsil[IDX(ti, tj)];
    double r_61 = p->sigma_2[IDX(ti, tj)] * inv_r_2;
    double r_6 = r_61 * r_61 * r_61;
    double r_12 = r_6 * r_6;
    *v_ff += l_eps * ((r_12 - r_6) - p->e_shift[IDX(ti, tj)]);
    double rd = l_eps * (-12 * r_12 + 6 * r_6) * inv_r_2;
    for (int d = 0; d < 3; ++d) {
      fi[d] -= rd * dr[d];
      force_tmp[3 * (j - 1) + d] += rd * dr[d];
    }
    {
      double f[3] = {-rd * dr[0], -rd * dr[1], -rd * dr[2]};
      vir_add(w, f, dr);
      /* scale: the repulsive and attractive parts before they cancel */
      const double m = fabs(l_eps) * (12 * r_12 + 6 * r_6) * inv_r_2 * sqrt(dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
      fsc_mag(o, i - 1, m);
      fsc_mag(o, j - 1, m);
    }
    int wall_pair = p->flags.wall == 1 && (ti == p->n_type - 1 || tj == p->n_type - 1);
    if (dpd && p->r_cut_dpd_2 == 0. && !wall_pair) { /* DPD inside the LJ range (dpd_forces.f90:45-53) */
      double w_r, w_d;
      if (p->flags.dpd_weight == 1) { w_r = w_d = 1.; } else {
        w_d = 1. - sqrt(r_2 * p->inv_range_2[IDX(ti, tj)]);
        w_r = w_d;
        w_d = w_d * w_d;
      }
      double g = orc_pair_gauss(o->s.seed, o->step, i - 1, j - 1);
      double ev[3], dv[3];
      for (int d = 0; d < 3; ++d) ev[d] = dr[d] * inv_sqrt_r_2;
      for (int d = 0; d < 3; ++d) dv[d] = o->v[3 * (i - 1) + d] - o->v[3 * (j - 1) + d];
      double rdot = dv[0] * ev[0] + dv[1] * ev[1] + dv[2] * ev[2];
      double fij[3];
      for (int d = 0; d < 3; ++d) {
        double fr = p->sig * w_r * g * ev[d];
        double fd = -1. * p->friction1 * w_d * rdot * ev[d];
        force_tmp[3 * (i - 1) + d] += fr + fd;
        force_tmp[3 * (j - 1) + d] -= fr + fd;
        fij[d] = fr + fd;
      }
      vir_add(w, fij, dr);
      dpd_scale(o, i, j, g);
    }
  }
  /* real-space Ewald (ewald_real.f90:15-33) */
  if (p->flags.system == 2 || p->flags.system == 3) {
    double qq = o->q[i - 1] * o->q[j - 1];
    int in_c = (p->compat & MFA_COMPAT_COUL_IN_LJ) || p->rc_coul_2 == 0. ? in_lj : (r_2_raw < p->rc_coul_2);
    if (in_c && qq != 0.) {
      double rc2 = in_lj ? r_2 : r_2_raw;
      double r = sqrt(rc2), inv_r = 1. / r;
      double erfcv = erfc(p->sqrt_alpha * r);
      *v_coul += qq * erfcv * inv_r;
      double fs = qq * p->sqrt_alpha * p->inv_sqrt_pi * 2. * exp(-p->alpha_c * rc2) * inv_r +
                  qq * erfcv * inv_r * inv_r;
      double fcv[3];
      for (int d = 0; d < 3; ++d) {
        double fc = fs * dr[d] * inv_r;
        force_tmp[3 * (i - 1) + d] += fc;
        if (!(p->compat & MFA_COMPAT_EWALD_I_ONLY)) force_tmp[3 * (j - 1) + d] -= fc;
        fcv[d] = fc;
      }
      vir_add(w, fcv, dr);
      fsc(o, i - 1, fcv);
      fsc(o, j - 1, fcv);
    }
  }
  /* DPD with its own cut-off (fluid_fluid.f90:217-258): heads excluded */
  if (dpd && p->r_cut_dpd_2 > 0.) {
    if (ti == 0 || tj == 0) return;
    if (p->flags.wall == 1 && (ti == p->n_type - 1 || tj == p->n_type - 1)) return;
    if (r_2 < p->r_cut_dpd_2) {
      double isr = 1. / sqrt(r_2);
      double w_r, w_d;
      if (p->flags.dpd_weight == 1) { w_r = w_d = 1.; } else {
        w_d = 1. - sqrt(r_2 / p->r_cut_dpd_2);
        w_r = w_d;
        w_d = w_d * w_d;
      }
      double g = orc_pair_gauss(o->s.seed, o->step, i - 1, j - 1);
      double ev[3], dv[3];
      for (int d = 0; d < 3; ++d) ev[d] = dr[d] * isr;
      for (int d = 0; d < 3; ++d) dv[d] = o->v[3 * (i - 1) + d] - o->v[3 * (j - 1) + d];
      double rdot = dv[0] * ev[0] + dv[1] * ev[1] + dv[2] * ev[2];
      double fij[3];
      for (int d = 0; d < 3; ++d) {
        double fr = p->sig * w_r * g * ev[d];
        double fd = -1. * p->friction1 * w_d * rdot * ev[d];
        force_tmp[3 * (i - 1) + d] += fr + fd;
        force_tmp[3 * (j - 1) + d] -= fr + fd;
        fij[d] = fr + fd;
      }
      vir_add(w, fij, dr);
      dpd_scale(o, i, j, g);
    }
  }
}

static void switch_on_r2min(orc_sys* o) {
  /* fluid_fluid.f90:35-42 */
  double r_time = (double)o->step * o->p.dt;
  if (o->p.flags.force_switch_on && r_time < o->p.r_2_min_time)
    o->r_2_min = (1. - r_time / o->p.r_2_min_time) * o->p.r_2_min_init;
  else
    o->r_2_min = 0.;
}

/* fluid_fluid() with BIN_TYPE 2 traversal (fluid_fluid.f90:71-477), serial. */
void orc_fluid_fluid(orc_sys* o) {
  switch_on_r2min(o);
  double vff = 0., vc = 0.;
  double* w = o->vir[0];
  memset(w, 0, 9 * sizeof(double));
  for (int ic = 1; ic <= o->nct; ++ic) {
    for (int i = o->part_in_cell[ic]; i != 0; i = o->r_nei[i]) {
      double fi[3] = {0, 0, 0};
      for (int jd = 0; jd < o->n_nei; ++jd) {
        int jc = o->cell_neigh_ls[(size_t)(ic - 1) * o->n_nei + jd];
        for (int j = o->part_in_cell[jc]; j != 0; j = o->r_nei[j]) pair_ij(o, i, j, fi, o->force, &vff, &vc, w);
      }
      for (int j = o->part_in_cell[ic]; j != 0; j = o->r_nei[j])
        if (i < j) pair_ij(o, i, j, fi, o->force, &vff, &vc, w);
      for (int d = 0; d < 3; ++d) o->force[3 * (i - 1) + d] += fi[d];
    }
  }
  if (o->p.flags.bin_type == 1) vff *= 0.5;
  o->v_ff = vff;
  o->v_coul = vc;
  if (o->p.flags.system == 2 || o->p.flags.system == 3) o->v_coul += o->v_coul_self;
}

/* The reference's OpenMP CPU path (fluid_fluid.f90:65-70,475-476): cells in static chunks of
 * 10, each thread a private force array, reduced at the end.  This is the timed CPU baseline. */
void orc_fluid_fluid_omp(orc_sys* o, int nthreads) {
  if (o->fscale) {  /* the force-scale accumulation is serial */
    orc_fluid_fluid(o);
    return;
  }
  switch_on_r2min(o);
  double vff = 0., vc = 0.;
  memset(o->vir[0], 0, 9 * sizeof(double));
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
  int nth = nthreads;
  size_t n3 = (size_t)3 * o->n;
  double* priv = (double*)calloc(n3 * nth, 8);
#pragma omp parallel num_threads(nth) reduction(+ : vff, vc)
  {
    int t = omp_get_thread_num();
    double* ft = priv + n3 * t;
    double wt[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma omp for schedule(static, 10)
    for (int ic = 1; ic <= o->nct; ++ic) {
      for (int i = o->part_in_cell[ic]; i != 0; i = o->r_nei[i]) {
        double fi[3] = {0, 0, 0};
        for (int jd = 0; jd < o->n_nei; ++jd) {
          int jc = o->cell_neigh_ls[(size_t)(ic - 1) * o->n_nei + jd];
          for (int j = o->part_in_cell[jc]; j != 0; j = o->r_nei[j]) pair_ij(o, i, j, fi, ft, &vff, &vc, wt);
        }
        for (int j = o->part_in_cell[ic]; j != 0; j = o->r_nei[j])
          if (i < j) pair_ij(o, i, j, fi, ft, &vff, &vc, wt);
        for (int d = 0; d < 3; ++d) ft[3 * (i - 1) + d] += fi[d];
      }
    }
#pragma omp critical
    for (int k = 0; k < 9; ++k) o->vir[0][k] += wt[k];
#pragma omp for schedule(static)
    for (size_t k = 0; k < n3; ++k) {
      double s = 0.;
      for (int u = 0; u < nth; ++u) s += priv[n3 * u + k];
      o->force[k] += s;
    }
  }
  free(priv);
  if (o->p.flags.bin_type == 1) vff *= 0.5;
  o->v_ff = vff;
  o->v_coul = vc;
  if (o->p.flags.system == 2 || o->p.flags.system == 3) o->v_coul += o->v_coul_self;
#else
  (void)nthreads;
  orc_fluid_fluid(o);
#endif
}

/* check_fluid_fluid (util.f90:284-330): O(N^2) total LJ energy over all n_part particles. */
double orc_check_fluid_fluid(orc_sys* o) {
  const mfa_params* p = &o->p;
  double vff = 0.;
  const double* L = o->s.boundary;
  for (int i = 0; i < o->n - 1; ++i) {
    int ti = o->a_type[i] - 1;
    for (int j = i + 1; j < o->n; ++j) {
      int tj = o->a_type[j] - 1;
      double dr[3];
      for (int d = 0; d < 3; ++d) dr[d] = o->r0[3 * i + d] - o->r0[3 * j + d];
      for (int d = 0; d < 2; ++d) dr[d] = dr[d] - L[d] * (double)(int64_t)(2 * dr[d] * (1. / L[d]));
      double r_2 = 0.;
      for (int d = 0; d < 3; ++d) r_2 += dr[d] * dr[d];
      if (r_2 < p->range_2[IDX(ti, tj)]) {
        if (r_2 < o->r_2_min) r_2 = o->r_2_min;
        double r_6 = ipow(p->sigma_2[IDX(ti, tj)] / r_2, 3);
        double r_12 = r_6 * r_6;
        vff += p->epsil[IDX(ti, tj)] * ((r_12 - r_6) - p->e_shift[IDX(ti, tj)]);
      }
    }
  }
  return vff;
}

/* All interacting pairs (0-based i<j) by O(N^2) search, same predicate as the pair kernel:
 * r^2 < range_2, or inside the DPD cut-off where DPD applies, or (charged) inside rc_coul. */
int64_t orc_pair_list(orc_sys* o, int32_t* pairs, int64_t cap) {
  const mfa_params* p = &o->p;
  const double* L = o->s.boundary;
  int64_t n = 0;
  for (int i = 0; i < o->nm - 1; ++i) {
    int ti = o->a_type[i] - 1;
    for (int j = i + 1; j < o->nm; ++j) {
      int tj = o->a_type[j] - 1;
      double dr[3];
      for (int d = 0; d < 3; ++d) dr[d] = o->r0[3 * i + d] - o->r0[3 * j + d];
      for (int d = 0; d < 2; ++d) dr[d] = dr[d] - L[d] * (double)(int64_t)(2 * dr[d] * (1. / L[d]));
      double r_2 = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
      int hit = r_2 < p->range_2[IDX(ti, tj)];
      if (!hit && p->flags.thermostat == 0 && p->r_cut_dpd_2 > 0. && ti != 0 && tj != 0 &&
          !(p->flags.wall == 1 && (ti == p->n_type - 1 || tj == p->n_type - 1)))
        hit = r_2 < p->r_cut_dpd_2;
      if (!hit && (p->flags.system == 2 || p->flags.system == 3) && p->rc_coul_2 > 0. &&
          !(p->compat & MFA_COMPAT_COUL_IN_LJ) && o->q[i] * o->q[j] != 0.)
        hit = r_2 < p->rc_coul_2;
      if (hit) {
        if (n < cap) { pairs[2 * n] = i; pairs[2 * n + 1] = j; }
        ++n;
      }
    }
  }
  return n;
}

/* fluid_wall(2) (fluid_wall.f90:77-125) */
void orc_fluid_wall(orc_sys* o) {
  const mfa_params* p = &o->p;
  double vfw = 0.;
  double D = o->s.boundary[2];
  memset(o->vir[5], 0, 9 * sizeof(double));
  if (p->flags.wall == 2) {
    for (int i = 0; i < o->nm; ++i) {
      int t = o->a_type[i] - 1;
      double z = o->r0[3 * i + 2];
      double inv_z = 1. / z;
      double rd = p->sigma_wall[t] * inv_z;
      double aw = fabs(p->a_wall[t]), sw = p->sigma_wall[t];
      vfw += aw * ipow(rd, 9) - p->a_w * ipow(rd, 3);
      const double f0 = o->force[3 * i + 2];
      o->force[3 * i + 2] += 9. * aw * ipow(sw, 9) * ipow(inv_z, 10);
      o->force[3 * i + 2] -= 3. * p->a_wall[t] * ipow(sw, 3) * ipow(inv_z, 4);
      const double fb = o->force[3 * i + 2] - f0;  /* the bottom wall's force */
      inv_z = 1. / (D - z);
      rd = sw * inv_z;
      vfw += aw * ipow(rd, 9) - p->a_w * ipow(rd, 3);
      const double f1 = o->force[3 * i + 2];
      o->force[3 * i + 2] -= 9. * aw * ipow(sw, 9) * ipow(inv_z, 10);
      o->force[3 * i + 2] += 3 * p->a_wall[t] * ipow(sw, 3) * ipow(inv_z, 4);
      const double ft = o->force[3 * i + 2] - f1;   /* the top wall's */
      /* each wall's force times the distance vector from the wall plane */
      o->vir[5][8] += fb * z + ft * (z - D);
      /* scale: both parts of each wall's force, times 10 (the force goes as z^-10, so a relative
         error of the distance is amplified tenfold) */
      fsc_mag(o, i, 10. * (9. * aw * ipow(sw, 9) * (ipow(1. / z, 10) + ipow(inv_z, 10)) +
                           3. * fabs(p->a_wall[t]) * ipow(sw, 3) * (ipow(1. / z, 4) + ipow(inv_z, 4))));
    }
  }
  o->v_fw = vfw;
}

/* wall_wall(2) (wall_wall.f90:45-48) */
void orc_wall_wall(orc_sys* o) {
  const mfa_params* p = &o->p;
  double D = o->s.boundary[2];
  o->v_ww = (p->flags.wall == 2)
                ? 2.0 * (fabs(p->a_w) * ipow(p->sigma_w / D, 9) - p->a_w * ipow(p->sigma_w / D, 3))
                : 0.;
}

static double fene_bond(orc_sys* o, int ip, int jp, int z_pbc) {
  /* intra_molec.f90:21-58 for the bond (ip, jp), 0-based */
  const mfa_params* p = &o->p;
  const double* L = o->s.boundary;
  double dr[3];
  for (int d = 0; d < 3; ++d) dr[d] = o->r0[3 * ip + d] - o->r0[3 * jp + d];
  for (int d = 0; d < 2 + z_pbc; ++d) dr[d] = dr[d] - L[d] * (double)(int64_t)(2. * dr[d] * (1. / L[d]));
  double r_2 = 0.;
  for (int d = 0; d < 3; ++d) r_2 += dr[d] * dr[d];
  double x = r_2 * p->inv_r_chain_2;
  if (x > (double)0.98f) x = (double)0.98f;
  double pot = -0.5 * log(1. - x);
  double rd = p->k_chain / (1. - x) * p->inv_r_chain_2;
  for (int d = 0; d < 3; ++d) {
    o->force[3 * ip + d] -= rd * dr[d];
    o->force[3 * jp + d] += rd * dr[d];
  }
  double f[3] = {-rd * dr[0], -rd * dr[1], -rd * dr[2]};  /* on ip; dr = r_ip - r_jp */
  vir_add(o->vir[1], f, dr);
  /* scale: the force over 1 - x (the condition of 1/(1 - x) near full stretch) */
  const double m = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]) / (1. - x);
  fsc_mag(o, ip, m);
  fsc_mag(o, jp, m);
  return pot;
}

/* intra_molec() (intra_molec.f90:16-188,266) */
void orc_intra_molec(orc_sys* o) {
  const mfa_system* s = &o->s;
  double vb = 0., vd = 0., ve = 0.;
  memset(o->vir[1], 0, 9 * sizeof(double));
  for (int c = 1; c <= s->n_chain; ++c)
    for (int m = 1; m <= s->n_mon - 1; ++m) {
      int ip = (c - 1) * s->n_mon + m;
      vb += fene_bond(o, ip - 1, ip, 0);
    }
  for (int c = 1; c <= s->n_chain_d; ++c)
    for (int m = 1; m <= s->n_mon_d - 1; ++m) {
      int ip = o->part_init_d + (c - 1) * s->n_mon_d + m;
      vd += fene_bond(o, ip - 1, ip, 0);
    }
  for (int c = 1; c <= s->n_chain_e; ++c)
    for (int m = 1; m <= s->n_mon_e - 1; ++m) {
      int ip = o->part_init_e + (c - 1) * s->n_mon_e + m;
      ve += fene_bond(o, ip - 1, ip, 0);
    }
  o->v_intra = o->p.k_chain * vb + o->p.k_chain * vd + o->p.k_chain * ve;
}

static void mic2(const orc_sys* o, double* r) {
  const double* L = o->s.boundary;
  r[0] = r[0] - L[0] * (double)(int64_t)(2. * r[0] * (1. / L[0]));
  r[1] = r[1] - L[1] * (double)(int64_t)(2. * r[1] * (1. / L[1]));
}

static double norm2v(const double* x) { return sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]); }

/* One bending term (bending.f90:30-109) for the triplet (a, b, c), 0-based, with r_prev =
 * r_b - r_a and r_next = r_c - r_b already min-imaged.  Returns the energy. */
static double bend_term(orc_sys* o, int ia, int ib, int ic, const double* r_prev, const double* r_next,
                        double k_b, double a_eq, int form, double* w) {
  double dot = 0, rp2 = 0, rn2 = 0, dp2 = 0, dn2 = 0;
  for (int j = 0; j < 3; ++j) {
    dot += r_next[j] * r_prev[j];
    rp2 += r_prev[j] * r_prev[j];
    rn2 += r_next[j] * r_next[j];
  }
  double cos_a = dot / sqrt(rp2 * rn2);
  double dn[3], dp[3];
  for (int j = 0; j < 3; ++j) {
    dn[j] = r_prev[j] * rn2 - r_next[j] * dot;
    dp[j] = -r_next[j] * rp2 + r_prev[j] * dot;
  }
  for (int j = 0; j < 3; ++j) { dp2 += dp[j] * dp[j]; dn2 += dn[j] * dn[j]; }
  const double small = (double)0.000001f;
  if (dn2 < small) {
    for (int j = 0; j < 3; ++j) dn[j] = r_prev[j] / sqrt(rp2) - r_next[j] / sqrt(rn2);
    dn2 = norm2v(dn);
    if (dn2 != 0.0) { for (int j = 0; j < 3; ++j) dn[j] = dn[j] / dn2 / sqrt(rn2); }
    else { for (int j = 0; j < 3; ++j) dn[j] = 0.; }
  } else {
    for (int j = 0; j < 3; ++j) dn[j] = dn[j] / sqrt(dn2 * rn2);
  }
  if (dp2 < small) {
    for (int j = 0; j < 3; ++j) dp[j] = r_prev[j] / sqrt(rp2) - r_next[j] / sqrt(rn2);
    dp2 = norm2v(dp);
    if (dp2 != 0.0) { for (int j = 0; j < 3; ++j) dp[j] = dp[j] / dp2 / sqrt(rp2); }
    else { for (int j = 0; j < 3; ++j) dp[j] = 0.; }
  } else {
    for (int j = 0; j < 3; ++j) dp[j] = dp[j] / sqrt(dp2 * rp2);
  }
  double fmod, e;
  if (form == 1) {
    /* cosine form V = k_b (1 - cos theta) with theta the bond angle from straight; dV/dtheta =
       k_b sin(theta), applied along the same unit directions as the harmonic form. */
    double th = (cos_a >= 1.0) ? 0. : acos(cos_a);
    fmod = k_b * sin(th);
    e = k_b * (1. - cos_a);
  } else {
    double da = (cos_a >= 1.0) ? 0. : acos(cos_a) - a_eq;
    fmod = k_b * da;
    e = .5 * fmod * da;
  }
  double fa[3], fc[3], fm[3], mrp[3];
  for (int j = 0; j < 3; ++j) {
    double fb0 = fmod * dp[j], fb1 = fmod * dn[j];
    o->force[3 * ia + j] += fb0;
    o->force[3 * ib + j] += -fb0 - fb1;
    o->force[3 * ic + j] += fb1;
    fa[j] = fb0; fc[j] = fb1; fm[j] = -fb0 - fb1; mrp[j] = -r_prev[j];
  }
  /* sum_k F_k (x) (r_k - r_b): r_a - r_b = -r_prev, r_c - r_b = r_next */
  vir_add(w, fa, mrp);
  vir_add(w, fc, r_next);
  fsc(o, ia, fa);
  fsc(o, ib, fa);  /* the centre bead's share: both parts */
  fsc(o, ib, fc);
  fsc(o, ic, fc);
  (void)fm;
  return e;
}

static double bend_chains(orc_sys* o, int beg, int n_chains, int n_mon, double* w) {
  double v = 0.;
  memset(w, 0, 9 * sizeof(double));
  for (int l = 0; l < n_chains; ++l) {
    int base = beg + l * n_mon; /* 0-based index of bead 1 */
    double r_next[3], r_prev[3];
    for (int d = 0; d < 3; ++d) r_next[d] = o->r0[3 * (base + 1) + d] - o->r0[3 * base + d];
    mic2(o, r_next);
    for (int i = 2; i <= n_mon - 1; ++i) {
      for (int d = 0; d < 3; ++d) r_prev[d] = r_next[d];
      for (int d = 0; d < 3; ++d) r_next[d] = o->r0[3 * (base + i) + d] - o->r0[3 * (base + i - 1) + d];
      mic2(o, r_next);
      v += bend_term(o, base + i - 2, base + i - 1, base + i, r_prev, r_next, o->p.k_bend, o->p.alpha_eq,
                     o->p.bend_form, w);
    }
  }
  return v;
}

/* bending(1) (bending.f90:19-121) */
void orc_bending(orc_sys* o) { o->v_bend = bend_chains(o, 0, o->s.n_chain, o->s.n_mon, o->vir[2]); }
/* bending_melt(1) (bending_melt.f90:22-108; the second index there lacks the `beg` offset, a
 * reference defect not reproduced: the consecutive melt bond is used). */
void orc_bending_melt(orc_sys* o) {
  o->v_bend_melt = bend_chains(o, o->part_init_d, o->s.n_chain_d, o->s.n_mon_d, o->vir[3]);
}

/* orientation(1) (orientation.f90:24-88) */
void orc_orientation(orc_sys* o) {
  double v = 0.;
  memset(o->vir[4], 0, 9 * sizeof(double));
  const double D = o->s.boundary[2];
  for (int l = 0; l < o->s.n_chain; ++l) {
    int h = l * o->s.n_mon; /* head, 0-based */
    double rg[3] = {o->r0[3 * h], o->r0[3 * h + 1], o->r0[3 * h + 2]};
    if (o->r0[3 * h + 2] > D / 2) rg[2] += 1.0; else rg[2] -= 1.0;
    double r_prev[3], r_next[3];
    for (int d = 0; d < 3; ++d) {
      r_prev[d] = o->r0[3 * h + d] - rg[d];
      r_next[d] = o->r0[3 * (h + 1) + d] - o->r0[3 * h + d];
    }
    mic2(o, r_next);
    mic2(o, r_prev);
    double dot = 0, rp2 = 0, rn2 = 0, dn2 = 0;
    for (int j = 0; j < 3; ++j) {
      dot += r_next[j] * r_prev[j];
      rp2 += r_prev[j] * r_prev[j];
      rn2 += r_next[j] * r_next[j];
    }
    double cos_a = dot / sqrt(rp2 * rn2);
    double dn[3];
    for (int j = 0; j < 3; ++j) dn[j] = r_prev[j] * rn2 - r_next[j] * dot;
    for (int j = 0; j < 3; ++j) dn2 += dn[j] * dn[j];
    if (dn2 < (double)0.000001f) {
      for (int j = 0; j < 3; ++j) dn[j] = r_prev[j] / sqrt(rp2) - r_next[j] / sqrt(rn2);
      dn2 = norm2v(dn);
      if (dn2 != 0.0) { for (int j = 0; j < 3; ++j) dn[j] = dn[j] / dn2 / sqrt(rn2); }
      else { for (int j = 0; j < 3; ++j) dn[j] = 0.; }
    } else {
      for (int j = 0; j < 3; ++j) dn[j] = dn[j] / sqrt(dn2 * rn2);
    }
    /* acos(cos_a >= 1) is NaN in the reference; the bending guard (bending.f90:93-98) is used */
    double da = ((cos_a >= 1.0) ? 0. : acos(cos_a)) - o->p.alpha_or;
    double fm = o->p.k_or * da;
    v += .5 * fm * da;
    double f1[3];
    for (int j = 0; j < 3; ++j) {
      o->force[3 * h + j] -= fm * dn[j];
      o->force[3 * (h + 1) + j] += fm * dn[j];
      f1[j] = fm * dn[j];
    }
    /* forces on the head and bead 1 only: F_1 (x) (r_1 - r_h) */
    vir_add(o->vir[4], f1, r_next);
    fsc(o, h, f1);
    fsc(o, h + 1, f1);
  }
  o->v_or = v;
}

/* constant_force(1) (constant_force.f90:17-21) */
void orc_constant_force(orc_sys* o) {
  for (int i = 0; i < o->nm; ++i) {
    for (int d = 0; d < 3; ++d) o->force[3 * i + d] += o->ext_force[3 * i + d];
    fsc(o, i, &o->ext_force[3 * i]);
  }
}

/* ewald_k(0) (ewald_k.f90:37-124) */
int orc_ewald_init(orc_sys* o) {
  const double pi = ref_pi();
  const double* L = o->s.boundary;
  double z_slab = 2.;
  double dk[3] = {2. * pi * (1. / L[0]), 2. * pi * (1. / L[1]), 2. * pi / (L[2] + z_slab * L[2])};
  double k_c = (dk[0] + dk[1]) * (double)o->p.n_kmax / 2.;
  int nx = (int)(k_c / dk[0]), ny = (int)(k_c / dk[1]), nz = (int)(k_c / dk[2]);
  int cap = (2 * nx + 1) * (2 * ny + 1) * (nz + 1);
  free(o->kv); free(o->k2); free(o->ik2);
  o->kv = (double*)malloc(sizeof(double) * 3 * cap);
  o->k2 = (double*)malloc(sizeof(double) * cap);
  o->ik2 = (double*)malloc(sizeof(double) * cap);
  int k = 0;
  for (int kz = 0; kz <= nz; ++kz)
    for (int ky = -ny; ky <= ny; ++ky)
      for (int kx = -nx; kx <= nx; ++kx) {
        double rk2 = ipow((double)kx * dk[0], 2) + ipow((double)ky * dk[1], 2) + ipow((double)kz * dk[2], 2);
        if (rk2 > k_c * k_c) continue;
        if (kz == 0 && ky == 0 && kx == 0) continue;
        if (kz == 0 && kx + ky < 0) continue;
        if (kz == 0 && -kx == ky && ky > 0) continue;
        o->kv[3 * k] = dk[0] * kx;
        o->kv[3 * k + 1] = dk[1] * ky;
        o->kv[3 * k + 2] = dk[2] * kz;
        o->k2[k] = o->kv[3 * k] * o->kv[3 * k] + o->kv[3 * k + 1] * o->kv[3 * k + 1] + o->kv[3 * k + 2] * o->kv[3 * k + 2];
        o->ik2[k] = 1. / o->k2[k];
        ++k;
      }
  o->nk = k;
  o->fac_alpha = 1. / (4. * o->p.alpha_c);
  o->inv_V_k = (1. / L[0]) * (1. / L[1]) / (L[2] * (1. + z_slab));
  return k;
}

int orc_ewald_kvecs(const orc_sys* o, double* out, int cap) {
  int n = o->nk < cap ? o->nk : cap;
  memcpy(out, o->kv, sizeof(double) * 3 * n);
  return o->nk;
}

/* ewald_k(1) (ewald_k.f90:128-202); returns u_cou_k and adds it to v_coul */
double orc_ewald_k(orc_sys* o) {
  const double pi = ref_pi();
  int nk = o->nk;
  double* re = (double*)calloc(nk, 8);
  double* im = (double*)calloc(nk, 8);
  for (int i = 0; i < o->nm; ++i) {
    if (o->q[i] == 0.) continue;
    for (int k = 0; k < nk; ++k) {
      double ph = o->kv[3 * k] * o->r0[3 * i] + o->kv[3 * k + 1] * o->r0[3 * i + 1] + o->kv[3 * k + 2] * o->r0[3 * i + 2];
      re[k] += o->q[i] * cos(ph);
      im[k] += o->q[i] * sin(ph);
    }
  }
  double u = 0.;
  memset(o->vir[6], 0, 9 * sizeof(double));
  for (int k = 0; k < nk; ++k) {
    const double uk = o->ik2[k] * exp(-o->k2[k] * o->fac_alpha) * (re[k] * re[k] + im[k] * im[k]);
    u += uk;
    /* reciprocal-space virial: u_k (delta_ab - 2 k_a k_b (1/k^2 + 1/(4 alpha_c))) */
    const double c = 2. * (o->ik2[k] + o->fac_alpha);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
        o->vir[6][3 * a + b] += uk * ((a == b ? 1. : 0.) - c * o->kv[3 * k + a] * o->kv[3 * k + b]);
  }
  u = u * 4. * pi * o->inv_V_k;
  for (int k = 0; k < 9; ++k) o->vir[6][k] *= 4. * pi * o->inv_V_k;
  for (int i = 0; i < o->nm; ++i) {
    if (o->q[i] == 0.) continue;
    double fk[3] = {0, 0, 0};
    for (int k = 0; k < nk; ++k) {
      double ph = o->kv[3 * k] * o->r0[3 * i] + o->kv[3 * k + 1] * o->r0[3 * i + 1] + o->kv[3 * k + 2] * o->r0[3 * i + 2];
      double s = o->ik2[k] * exp(-o->k2[k] * o->fac_alpha) * (cos(ph) * im[k] - sin(ph) * re[k]);
      for (int d = 0; d < 3; ++d) fk[d] += o->kv[3 * k + d] * s;
    }
    double fkv[3];
    for (int d = 0; d < 3; ++d) {
      fkv[d] = -8. * pi * o->q[i] * fk[d] * o->inv_V_k;
      o->force[3 * i + d] += fkv[d];
    }
    fsc(o, i, fkv);
  }
  free(re);
  free(im);
  o->v_coul += u;
  return u;
}

/* dipolar_correction (dipolar_correction.f90:20-33); uses the slab volume of ewald_k(0) */
double orc_dipolar_correction(orc_sys* o) {
  const double pi = ref_pi();
  double mz = 0.;
  for (int i = 0; i < o->nm; ++i) mz += o->q[i] * (o->r0[3 * i + 2] - o->lz_half);
  for (int i = 0; i < o->nm; ++i) {
    o->force[3 * i + 2] -= 4. * pi * o->q[i] * mz * o->inv_V_k;
    fsc_mag(o, i, 4. * pi * o->q[i] * mz * o->inv_V_k);
  }
  double u = 2. * pi * mz * mz * o->inv_V_k;
  /* minus the strain derivative of u (M_z scales with z, the volume with each axis):
     diag(u, u, -u) */
  memset(o->vir[7], 0, 9 * sizeof(double));
  o->vir[7][0] = u;
  o->vir[7][4] = u;
  o->vir[7][8] = -u;
  o->v_coul += u;
  return u;
}

/* verlet_positions (verlet_positions.f90:150-209, BIN_TYPE 2, SYMMETRY 0) */
void orc_verlet_positions(orc_sys* o) {
  const double dt = o->p.dt, dt_2 = dt * dt;
  const double* L = o->s.boundary;
  for (int i = 1; i <= o->nm; ++i) {
    double* r = &o->r0[3 * (i - 1)];
    double* v = &o->v[3 * (i - 1)];
    double* a = &o->a[3 * (i - 1)];
    int old_cell = get_cell(o, r);
    for (int d = 0; d < 3; ++d) r[d] = r[d] + dt * v[d] + 0.5 * dt_2 * a[d];
    for (int d = 0; d < 2; ++d) {
      if (r[d] > L[d]) r[d] = r[d] - L[d];
      else if (r[d] < 0.) r[d] = r[d] + L[d];
    }
    update_part_cell(o, i, old_cell);
    for (int d = 0; d < 3; ++d) v[d] = v[d] + 0.5 * dt * a[d];
  }
  /* verlet_positions.f90:214-247 (WALL 1 with a wall velocity): the sites of wall beads
     1..n_wall/2 move by +va_spring_twall dt, the others by -va_spring_twall dt, wrapped into
     [0, L) in x and y, and the beads sit on their sites (their velocity stays 0).  Their cells
     follow them here (the reference's linked cells hold the mobile particles only). */
  if (o->p.flags.wall == 1 && (o->p.va_wall[0] != 0. || o->p.va_wall[1] != 0.)) {
    const int n_wall = o->n - o->nm;
    for (int k = 0; k < n_wall; ++k) {
      const int i = o->nm + 1 + k;
      double* r = &o->r0[3 * (i - 1)];
      const int old_cell = get_cell(o, r);
      for (int d = 0; d < 2; ++d) {
        const double dd = o->p.va_wall[d] * dt;
        r[d] = (k < n_wall / 2) ? r[d] + dd : r[d] - dd;
        if (r[d] > L[d]) r[d] = r[d] - L[d];
        else if (r[d] < 0.) r[d] = r[d] + L[d];
      }
      update_part_cell(o, i, old_cell);
    }
  }
}

/* verlet_velocities (verlet_velocities.f90:25-178) */
void orc_verlet_velocities(orc_sys* o) {
  const double dt = o->p.dt;
  /* f_on_heads (verlet_velocities.f90:18), summed as fort.80 writes it (observation.f90:324-327) */
  for (int k = 0; k < 6; ++k) o->f_heads[k] = 0.;
  for (int c = 0; c < o->s.n_chain; ++c) {
    const int h = c * o->s.n_mon, half = (c < o->s.n_chain / 2) ? 0 : 3;
    for (int d = 0; d < 3; ++d) o->f_heads[half + d] -= o->force[3 * h + d];
  }
  for (int i = 0; i < o->nm; ++i)
    for (int d = 0; d < 3; ++d) {
      o->a[3 * i + d] = o->force[3 * i + d] * o->inv_mass[i];
      o->v[3 * i + d] = o->v[3 * i + d] + 0.5 * dt * o->a[3 * i + d];
    }
  if (o->p.flags.poiseuille) {
    for (int c = 0; c < o->s.n_chain; ++c) {
      int h = c * o->s.n_mon;
      for (int d = 0; d < 3; ++d) o->v[3 * h + d] = o->force[3 * h + d] = o->a[3 * h + d] = 0.;
    }
  } else {
    /* verlet_velocities.f90:111-124: the heads of chains 1..n_chain/2 move at va_spring_twall(1:2),
       the others at -va_spring_twall(1:2); no z velocity, force or acceleration */
    for (int c = 0; c < o->s.n_chain; ++c) {
      int h = c * o->s.n_mon;
      const double sg = (c < o->s.n_chain / 2) ? 1. : -1.;
      for (int d = 0; d < 3; ++d) o->force[3 * h + d] = o->a[3 * h + d] = 0.;
      o->v[3 * h] = sg * o->p.va_wall[0];
      o->v[3 * h + 1] = sg * o->p.va_wall[1];
      o->v[3 * h + 2] = 0.;
    }
  }
  double t = 0.;
  for (int i = 0; i < o->nm; ++i)
    t += o->mass[i] * (o->v[3 * i] * o->v[3 * i] + o->v[3 * i + 1] * o->v[3 * i + 1] + o->v[3 * i + 2] * o->v[3 * i + 2]);
  o->t_fluid = 0.5 * t;
}

/* histo(2) + velocity_prof(2) (functions.f90:157-214, 319-365) */
void orc_profiles_accumulate(orc_sys* o) {
  int H = o->hist;
  double inv_z_step = 1. / (o->s.boundary[2] / (double)H);
  o->n_obs++;
  for (int i = 0; i < o->nm; ++i) {
    int sp = (i < o->part_init_d) ? 0 : (i < o->part_init_e ? 1 : 2);
    int zi = (int)(o->r0[3 * i + 2] * inv_z_step) + 1;
    if (zi < 1) zi = 1;
    if (zi > H) zi = H;
    zi -= 1;
    o->dens[zi * 3 + sp] += 1.;
    for (int d = 0; d < 3; ++d) {
      double vv = o->v[3 * i + d];
      o->vp[(zi * 3 + sp) * 3 + d] += vv;
      o->vp2[(zi * 3 + sp) * 3 + d] += vv * vv;
    }
  }
}

int64_t orc_get_profiles(const orc_sys* o, double* dens, double* vs, double* v2) {
  int H = o->hist;
  if (dens) memcpy(dens, o->dens, sizeof(double) * H * 3);
  if (vs) memcpy(vs, o->vp, sizeof(double) * H * 9);
  if (v2) memcpy(v2, o->vp2, sizeof(double) * H * 9);
  return o->n_obs;
}

/* Force routines of md_main.f90:107-171 on the current positions and velocities. */
void orc_forces(orc_sys* o, int nthreads) {
  const mfa_flags* f = &o->p.flags;
  orc_zero_force(o);
  if (nthreads > 1) orc_fluid_fluid_omp(o, nthreads); else orc_fluid_fluid(o);
  orc_fluid_wall(o);
  orc_wall_wall(o);
  orc_intra_molec(o);
  if (f->bending) orc_bending(o);
  if (f->bending_melt) orc_bending_melt(o);
  if (f->orientation) orc_orientation(o);
  if (f->system == 2 || f->system == 3) {
    if (o->nk == 0) orc_ewald_init(o);
    orc_ewald_k(o);
    orc_dipolar_correction(o);
  }
  if (f->poiseuille) orc_constant_force(o);
}

/* nsteps iterations of md_main.f90:77-202 (profiles every step when `profiles`). */
void orc_step(orc_sys* o, int nsteps, int nthreads, int profiles) {
  for (int it = 0; it < nsteps; ++it) {
    o->i_time++;
    orc_verlet_positions(o);
    orc_forces(o, nthreads);
    orc_verlet_velocities(o);
    if (profiles) orc_profiles_accumulate(o);
    o->step++;
  }
}

int orc_n_kvec(const orc_sys* o) { return o->nk; }
