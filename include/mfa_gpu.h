/*
 * mfa_gpu.h -- C ABI of the GB300 (sm_103a) MD-DPD step for polymer brushes in a slit channel.
 *
 * This library is a drop-in for the per-timestep hot path of mfa_brush ("MFA_PROG"), the Fortran
 * molecular-dynamics code whose main loop is md_main.f90:77-215.  Each entry point below replaces
 * one argument-less subroutine that md_main calls (cited per function).  The Fortran module
 * `commons` (mfa_common.f90) holds the state as column-major (3,N) REAL(8) arrays, i.e. AoS xyz
 * doubles; the same layout is used here for every host array: r0[3*i+d], v[3*i+d], a[3*i+d].
 * Particle types are the reference's 1-based a_type values.
 *
 * Ownership: the library copies the host state to the device once (mfa_init / mfa_batch_init),
 * keeps it resident in HBM and only copies back on mfa_sync_to_host, mfa_get_* or when an entry
 * point is given a non-NULL energy pointer.  All calls on one context are issued on one CUDA
 * stream and are asynchronous unless they return host data.  A context is not thread-safe.
 *
 * Errors: every entry point returns MFA_OK (0) or a negative MFA_ERR_* status and never aborts,
 * traps or exits; mfa_last_error() gives a one-line description.  The reference instead prints
 * and STOPs (e.g. init_system.f90:135-137, cell_list.f90:406-407).
 *
 * Batching: a context holds R >= 1 independent replicas ("systems") that share one parameter
 * set (type tables, thermostat, bonded constants) but each has its own box, chain counts, particle
 * count and noise seed.  Particles of all replicas are concatenated replica-major in every host
 * array.  mfa_init is mfa_batch_init with R = 1.
 */
#ifndef MFA_GPU_H
#define MFA_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MFA_MAX_TYPES 6
#define MFA_HIST_DIM_MAX 1024

/* ---- status codes ---------------------------------------------------------------------- */
#define MFA_OK 0
#define MFA_ERR_ARG (-1)             /* invalid argument / size                               */
#define MFA_ERR_CUDA (-2)            /* a CUDA runtime call failed                             */
#define MFA_ERR_ALLOC (-3)           /* device or host allocation failed                       */
#define MFA_ERR_NLIST_OVERFLOW (-4)  /* a particle has more neighbours than the list holds     */
#define MFA_ERR_OUT_OF_BOX (-5)      /* a particle left the channel (z < -l_cell or z > D+l)   */
#define MFA_ERR_NAN (-6)             /* non-finite position/velocity detected                  */
#define MFA_ERR_IO (-7)              /* file could not be opened / read                        */
#define MFA_ERR_PARSE (-8)           /* malformed input file                                   */
#define MFA_ERR_UNSUPPORTED (-9)     /* option combination not built                           */
#define MFA_ERR_NO_DEVICE (-10)      /* no CUDA device visible                                 */
#define MFA_ERR_STATE (-11)          /* entry point called in the wrong order                  */
#define MFA_ERR_CAPACITY (-12)       /* request exceeds a fixed, documented maximum            */

/* ---- precision modes ------------------------------------------------------------------- */
#define MFA_PREC_FP64 0   /* plain FP64: every pair/bond/integration operation in double     */
#define MFA_PREC_MIXED 1  /* FP32 pair/bond arithmetic on fixed-point positions, FP32 per-pair
                             accumulation, FP64 per-particle totals, FP64 integration and
                             FP64 energy reductions                                           */

/* ---- reference-defect reproduction switches (mfa_params.compat bit mask) ---------------- */
#define MFA_COMPAT_EWALD_INV_PI 1u     /* inv_sqrt_pi = 1/pi (init_config.f90:232)               */
#define MFA_COMPAT_EWALD_I_ONLY 2u     /* real-space Coulomb force on i only (ewald_real.f90:30) */
#define MFA_COMPAT_COUL_IN_LJ 4u       /* real-space Coulomb only inside the LJ cut-off
                                          (fluid_fluid.f90:121,203-209)                          */

/*
 * Compile-time macros of control_simulation.h (control_simulation.h:9-105) as run-time options.
 * Only the values listed are built; others make mfa_derive_params return MFA_ERR_UNSUPPORTED.
 */
typedef struct mfa_flags {
  int32_t system;           /* SYSTEM: 0 brush channel, 2 charged (no brush), 3 charged + brush */
  int32_t symmetry;         /* SYMMETRY: 0 (channel, walls in z)                                 */
  int32_t wall;             /* WALL: 1 explicit wall beads, 2 implicit 9-3 walls                 */
  int32_t solvent;          /* SOLVENT 0..3 (cut-off/shift table rules, init_params.f90:497-737) */
  int32_t hydrophobia;      /* HYDROPHOBIA                                                       */
  int32_t brush_in_good_sv; /* BRUSH_IN_GOOD_SV                                                  */
  int32_t bending;          /* BENDING (brush chains)                                            */
  int32_t bending_melt;     /* BENDING_MELT (melt chains)                                        */
  int32_t orientation;      /* ORIENTATION (head ghost-bond stiffness)                           */
  int32_t particle_4;       /* PARTICLE_4                                                        */
  int32_t thermostat;       /* THERMOSTAT: 0 DPD, 1 Langevin (its call is commented out in the
                               reference, fluid_fluid.f90:455-458, so: no thermostat)            */
  int32_t dpd_weight;       /* DPD_WEIGHT: 0 (w_R = 1-r/rc, w_D = w_R^2), 1 (w = 1)             */
  double dpd_cut_off;       /* DPD_CUT_OFF value, 0 = macro undefined                            */
  int32_t force_switch_on;  /* FORCE_SWITCH_ON                                                   */
  int32_t poiseuille;       /* POISEUILLE (constant body force, heads held fixed)                */
  int32_t profiles;         /* PROFILES                                                          */
  int32_t bin_type;         /* BIN_TYPE 0/1/2: changes only the energy bookkeeping here          */
  int32_t l_box;            /* L_BOX 1 (l_cell >= r_cut_max, 13 cells) or 2 (r_cut_max/2, 62)   */
  int32_t free_heads;       /* FREE_HEADS (not built: must be 0)                                 */
  int32_t sheared;          /* SHEARED (not built: must be 0)                                    */
} mfa_flags;

/* Raw values of system_input (init_system.f90:16-138) and mfa_input (init_params.f90:141-244). */
typedef struct mfa_inputs {
  mfa_flags flags;
  /* system_input */
  int32_t n_mon, n_chain, n_cell_w_x, n_cell_w_y;
  int32_t n_mon_d, n_chain_d;
  double drop_cell_x, drop_cell_y, z_skin;
  int32_t n_mon_e, n_chain_e, inter4;
  double delta_sig[3];
  double a_w, sigma_w, a_w4, sigma_w4;
  double charge[MFA_MAX_TYPES];
  double alpha_c;
  int32_t n_kmax;
  double const_force[3];
  /* mfa_input */
  int64_t s_time, n_relax, n_obser, n_safe;
  double dt, temp, x_space, y_space, z_space_wall;
  double mass_type[MFA_MAX_TYPES];
  double epsil[MFA_MAX_TYPES * MFA_MAX_TYPES]; /* row-major [i*MAX+j], 0-based types            */
  double sigma_ii[MFA_MAX_TYPES];
  double friction[MFA_MAX_TYPES];
  double k_spring_wall, k_bend, alpha_eq;
  int64_t iseed;
  double k_chain, r_chain;
  int32_t f_twall[3];
  double va_spring_twall[3], k_spring_twall[3];
  /* extensions that the reference cannot express (0 = reference behaviour) */
  int32_t bend_form;        /* 0 harmonic in angle (bending.f90:97-100), 1 cosine k_b(1-cos)   */
  double rc_coul;           /* own real-space Coulomb cut-off (0: LJ cut-off, fluid_fluid.f90:203) */
  uint32_t compat;          /* MFA_COMPAT_* bits                                                */
  int32_t hist_dim;         /* z-profile bins (init_obser.f90:120 uses 200)                     */
} mfa_inputs;

/* Derived, shared physics parameters (restatement of init_params.f90:393-887). */
typedef struct mfa_params {
  mfa_flags flags;
  int32_t n_type;
  double dt, temp;
  double mass_type[MFA_MAX_TYPES];
  double epsil[MFA_MAX_TYPES * MFA_MAX_TYPES];       /* 4*eps (init_params.f90:468)            */
  double sigma[MFA_MAX_TYPES * MFA_MAX_TYPES];
  double sigma_2[MFA_MAX_TYPES * MFA_MAX_TYPES];
  double range_2[MFA_MAX_TYPES * MFA_MAX_TYPES];     /* LJ cut-off squared, 0 = no interaction */
  double inv_range_2[MFA_MAX_TYPES * MFA_MAX_TYPES];
  double e_shift[MFA_MAX_TYPES * MFA_MAX_TYPES];
  double r_cut_max;                                  /* init_params.f90:792-808               */
  double r_cut_dpd_2;                                /* DPD_CUT_OFF^2, 0 if undefined          */
  double friction1;                                  /* gamma = friction(1)                    */
  double sig;                                        /* sqrt(2 kT gamma / dt)                  */
  double sigma_wall[MFA_MAX_TYPES], a_wall[MFA_MAX_TYPES];
  double a_w, sigma_w;
  double k_chain;                                    /* k*R0^2 (init_params.f90:396)           */
  double r_chain_2, inv_r_chain_2;
  double k_bend, alpha_eq, k_or, alpha_or;
  int32_t bend_form;
  double const_force[3];
  double charge[MFA_MAX_TYPES];
  double alpha_c, sqrt_alpha, inv_sqrt_pi;
  int32_t n_kmax;
  double rc_coul_2;                                  /* 0: Coulomb inside the LJ cut-off       */
  double skin;                                       /* Verlet skin of BIN_TYPE 0 (0.4f)       */
  double r_2_min_init, r_2_min_time;                 /* force switch-on ramp                   */
  uint32_t compat;
  int32_t hist_dim;
  double va_wall[2];        /* x, y velocity of the heads of chains 1..n_chain/2, the other heads
                               moving at -va_wall (verlet_velocities.f90:111-124: the two brushes
                               sheared against each other); with explicit walls (WALL 1) also the
                               sites of wall beads 1..n_wall/2 (the others at -va_wall,
                               verlet_positions.f90:214-247); mfa_inputs.va_spring_twall(1:2).
                               0 without shear; the reference stops on a non-zero value with
                               POISEUILLE (init_params.f90:899-907)                             */
} mfa_params;

/* Per-replica geometry and topology. */
typedef struct mfa_system {
  double boundary[3];       /* Lx, Ly, D (init_config.f90:11-22)                               */
  int32_t n_mon, n_chain;   /* brush: n_chain chains of n_mon beads, heads at (c-1)*n_mon+1   */
  int32_t n_mon_d, n_chain_d; /* melt/solvent chains following the brush                      */
  int32_t n_mon_e, n_chain_e; /* particle-4 chains following the melt                         */
  int32_t n_mon_tot;        /* mobile particles                                                 */
  int32_t n_part;           /* n_mon_tot + explicit wall beads                                  */
  int64_t s_time;           /* starting step (mfa_input line 1)                                 */
  uint64_t seed;            /* key of this replica's DPD noise stream                           */
} mfa_system;

typedef struct mfa_options {
  int32_t precision;        /* MFA_PREC_FP64 or MFA_PREC_MIXED                                  */
  int32_t device;           /* CUDA device ordinal                                              */
  double skin;              /* neighbour-list skin in sigma (default 0.3)                       */
  int32_t nbr_capacity;     /* neighbours per particle; 0 = estimate from density and cut-off  */
  int32_t energy_every;     /* steps between energy reductions in mfa_step (10, as fort.60)     */
  int32_t use_graphs;       /* capture mfa_step sequences as CUDA graphs (default 1)            */
  int32_t block_size;       /* threads per block of the pair kernel: 32, 64 or 128; other
                               values (0) take the built-in 128                                 */
  int32_t profile_from_step;/* mfa_step accumulates z-profiles for steps > this (n_relax)       */
  int32_t kspace_plain_sums;/* 1: mixed-precision k-space sums in plain FP32, without the Kahan
                               compensation across particle tiles and k rows (a precision study;
                               default 0)                                                       */
  int32_t observe;          /* 1: mfa_step adds every energy record of the steps after
                               profile_from_step (n_relax) to the observation averages
                               (mfa_get_averages); default 0                                    */
  int32_t series_capacity;  /* energy records kept on the device for mfa_get_energy_series (a
                               ring; 0 = none, the default)                                     */
  int32_t list_cells;       /* list-build cells per list cut-off (r_cut_max + skin) along each
                               axis: 1, 2 or 3; 0 (the default) = the smallest value for which
                               every box holds 2*list_cells+1 cells in x and y.  The list search
                               walks the (2*list_cells+1)^3 cells around a particle as x-rows and
                               skips the rows and row ends beyond the cut-off.  The lists hold the
                               same pairs whatever the value; their order differs.               */
  int32_t pair_schedule;    /* 0 (default): the pair kernel runs one block per 128 particles;
                               1: as many blocks as fit on the GPU at once, each taking blocks of
                               particles from a queue (an atomic ticket, no waiting) until none
                               is left.  The forces are the same bit for bit.                    */
  int32_t separate_integrator; /* 0 (default): in the mixed-precision mfa_step without k-space,
                               the steps without an energy record run their integration in the
                               tail of the pair kernel (one launch per step instead of two);
                               1: a separate integrator kernel on every step.  The trajectory is
                               the same bit for bit.                                          */
  int32_t list_cells_x;     /* list-build cells per list cut-off along x alone: 1, 2 or 3 when
                               list_cells is 1 (finer cells in x trim the x-runs of the 3x3 rows
                               closer to the cut-off sphere); 0 (default) = 2 when list_cells is
                               1 and every box holds 5 such cells in x, else list_cells        */
} mfa_options;

typedef struct mfa_energies {
  int64_t step;             /* absolute step of this record                                     */
  double v_fluid_fluid, v_fluid_wall, v_wall_wall, v_intra_molec;
  double v_bend, v_bend_melt, v_or, v_coul;
  double t_fluid;           /* 0.5 sum m v^2 over mobile particles (verlet_velocities.f90:132) */
  double v_total, e_total;  /* verlet_velocities.f90:155-178                                   */
  double inv_n;             /* 1/(n_mon_tot - n_chain) (init_params.f90:479-481)              */
} mfa_energies;

/* Observation quantities of one replica (observation.f90 and verlet_velocities.f90:18). */
typedef struct mfa_observables {
  int64_t step;             /* absolute step of the positions and velocities used               */
  double rg2_brush[3];      /* mean over brush chains of the per-axis Rg^2, chains unfolded bond
                               by bond (observation.f90:187-201,214-245)                        */
  double rg2_melt[3];       /* the same over the melt chains (observation.f90:262-272; chains
                               counted from the first melt particle)                            */
  double momentum[3];       /* sum of m v over the mobile particles (observation.f90:286-291)   */
  double f_heads[2][3];     /* minus the summed force on the heads of chains 1..n_chain/2 and of
                               the other chains, at the last energy record (verlet_velocities.f90:18,
                               observation.f90:324-327)                                          */
} mfa_observables;

/* Virial and pressure tensors of one replica (the reference's press_tensor, fluid_fluid.f90:156-166,
   dpd_forces.f90:118-127, intra_molec.f90:60-67, viscosity.f90:20-33, obser_out.f90:309-318).
   Every tensor is row-major, w[3 a + b].  A group's virial is minus the derivative of its energy
   under the strain r_a -> r_a + e r_b of positions and box: for pair, bond and angle terms the sum
   over the terms of F_a (r_i - r_j)_b with F the force on particle i (the sign of the reference's
   pair term; its brush-bond term, intra_molec.f90:64, has the opposite sign, which is not
   reproduced), for the walls each wall's force times the distance from its plane, for the
   reciprocal-space and slab-dipole energies the derivative of their volume-dependent sums.
   The pair group holds LJ, DPD (random and dissipative) and real-space Coulomb; the body force
   of POISEUILLE has no virial.                                                              */
typedef struct mfa_virial {
  int64_t step;             /* absolute step of the record                                      */
  double pair[9], fene[9], bend[9], bend_melt[9], orientation[9], wall[9], kspace[9], dipole[9];
  double total[9];          /* sum of the groups                                                */
  double kinetic[9];        /* sum of m v_a v_b over the mobile particles (viscosity.f90:20-27) */
  double volume;            /* Lx Ly D                                                          */
  double pressure[9];       /* (kinetic + total) / volume                                       */
} mfa_virial;

/* Time averages of the observation phase of one replica (observation.f90:17-291, written to
   fort.40, fort.42 and fort.43 by observation.f90:295-314 and to the pressure block by
   obser_out.f90:309-318): sums over the observations divided by their number.              */
typedef struct mfa_averages {
  int64_t count;            /* observations summed (count_obs)                                  */
  double v_total, t_total, e_total;        /* means (fort.40; t_total = t_fluid)               */
  double v_total2, t_total2, e_total2;     /* means of their squares                           */
  double v_fluid, t_fluid, e_fluid;        /* v_ff + v_intra + v_fw, t_fluid, v_ff + t_fluid
                                              (observation.f90:150-157)                        */
  double v_fluid2, t_fluid2, e_fluid2;
  double momentum[3];       /* tot_P / count_obs (fort.40)                                       */
  double rg2_brush[3], rg2_melt[3], rg2_mean[3];  /* r_g2_mean(1..3,:) / count_obs (fort.42)    */
  double r_par_per2[2];     /* brush and melt (Rg_z^2 - (Rg_x^2 + Rg_y^2)/2) / Rg^2 (fort.43)     */
  double pressure[9];       /* press_tensor_mean / count_obs: the mean of mfa_virial.pressure   */
  double f_heads[2][3];     /* the mean of mfa_observables.f_heads: minus the summed force on the
                               heads of chains 1..n_chain/2 and of the others (the f_on_heads of
                               obser_out.f90:160-176, whose x component over twice the wall area
                               is the shear stress, and times D / va_spring_twall(1) the
                               effective viscosity of the sheared brushes)                     */
} mfa_averages;

typedef struct mfa_ctx mfa_ctx;

/* ---- library / device ------------------------------------------------------------------ */
const char* mfa_version(void);
int mfa_device_count(int32_t* n);
void mfa_default_options(mfa_options* opt);

/* ---- host-side input handling ---------------------------------------------------------- */
/* Parses #define/#undef lines of a control_simulation.h (replaces the cpp step of Makefile:8). */
int mfa_flags_from_header(const char* path, mfa_flags* out);
/* init_system.f90:16-138: reads system_input with the layout that io->flags selects. */
int mfa_read_system_input(const char* path, mfa_inputs* io);
/* init_params.f90:141-244: reads mfa_input. */
int mfa_read_mfa_input(const char* path, mfa_inputs* io);
/* init_params.f90:393-887 + init_config.f90:11-22,219-241: derived tables and the box. */
int mfa_derive_params(const mfa_inputs* in, mfa_params* out, mfa_system* sys_out);
/* init_config.f90:109-208: conf_old reader (types, positions, velocities, accelerations). */
int mfa_read_conf_old(const char* path, int32_t n_part, int32_t* a_type, double* r0, double* v,
                      double* a);
/* store_config.f90:14-63 (case 2): conf_new writer.  With in->flags.wall == 1 the explicit wall
   beads (the particles after the mobile ones) are written as the r_wall_equi block
   (store_config.f90:47-52); the top/bottom wall block is zero (the walls do not move).        */
int mfa_write_conf_new(const char* path, const mfa_inputs* in, int32_t n_part,
                       const int32_t* a_type, const double* r0, const double* v, const double* a);
/* init_force_switch_on.f90:12-28: sets r_2_min_init/r_2_min_time of p (used when s_time == 1). */
int mfa_force_switch_on(mfa_params* p, int64_t n_relax, int64_t n_obser);

/* ---- context --------------------------------------------------------------------------- */
/* On a failure after the context was made (every status but MFA_ERR_ARG and MFA_ERR_NO_DEVICE),
   *out still holds it so that mfa_last_error(*out) can say why; release it with mfa_destroy.   */
int mfa_init(const mfa_params* p, const mfa_system* sys, const int32_t* a_type, const double* r0,
             const double* v, const double* a, const mfa_options* opt, mfa_ctx** out);
int mfa_batch_init(const mfa_params* p, int32_t n_rep, const mfa_system* sys,
                   const int32_t* a_type, const double* r0, const double* v, const double* a,
                   const mfa_options* opt, mfa_ctx** out);
int mfa_destroy(mfa_ctx* ctx);
const char* mfa_last_error(const mfa_ctx* ctx);
int mfa_synchronize(mfa_ctx* ctx);
/* The context's cudaStream_t (as void*), for callers that order their own work after it. */
void* mfa_stream(mfa_ctx* ctx);
int mfa_n_particles(const mfa_ctx* ctx, int64_t* n_total, int32_t* n_rep);

/* ---- per-routine drop-ins (md_main.f90:85-185 order) -------------------------------------
 * Energy out-pointers are optional: NULL keeps the call asynchronous; non-NULL synchronises
 * and returns one value per replica (an array of n_rep doubles).                             */
/* verlet_positions.f90:150-209: r += dt v + dt^2/2 a, wrap x,y, v += dt/2 a; then the cell /
   neighbour-list update that the reference does in update_part_cell (cell_list.f90:215-268). */
int mfa_verlet_positions(mfa_ctx* ctx);
/* check_skin.f90:11-24 + binning.f90: rebuilds the lists if any particle moved > skin/2. */
int mfa_check_skin(mfa_ctx* ctx, int32_t* rebuilt);
/* md_main.f90:107 force(:,:) = 0. */
int mfa_zero_force(mfa_ctx* ctx);
/* fluid_fluid.f90:1-512 with dpd_forces.f90 and ewald_real.f90 fused: adds pair forces. */
int mfa_fluid_fluid(mfa_ctx* ctx, double* v_fluid_fluid, double* v_coul);
/* fluid_wall.f90:77-125 (wall_type 2). */
int mfa_fluid_wall(mfa_ctx* ctx, int32_t wall_type, double* v_fluid_wall);
/* wall_wall.f90:45-48. */
int mfa_wall_wall(mfa_ctx* ctx, int32_t wall_type, double* v_wall_wall);
/* intra_molec.f90:16-129 (FENE: brush, melt, particle-4 chains). */
int mfa_intra_molec(mfa_ctx* ctx, double* v_intra_molec);
/* bending.f90:19-121 (mode 1). */
int mfa_bending(mfa_ctx* ctx, int32_t mode, double* v_bend);
/* bending_melt.f90:22-108 (mode 1). */
int mfa_bending_melt(mfa_ctx* ctx, int32_t mode, double* v_bend_melt);
/* orientation.f90:24-88 (mode 1). */
int mfa_orientation(mfa_ctx* ctx, int32_t mode, double* v_or);
/* ewald_k.f90:128-202 (mode 1; mode 0 = set-up, done at init). */
int mfa_ewald_k(mfa_ctx* ctx, int32_t mode, double* v_coul_k);
/* dipolar_correction.f90:20-33. */
int mfa_dipolar_correction(mfa_ctx* ctx, double* v_dip);
/* constant_force.f90:16-21 (mode 1). */
int mfa_constant_force(mfa_ctx* ctx, int32_t mode);
/* verlet_velocities.f90:14-178: a = F/m, v += dt/2 a, head constraints, energies. */
int mfa_verlet_velocities(mfa_ctx* ctx, mfa_energies* e);
/* functions.f90:157-214,319-365: histo(2) + velocity_prof(2) on the current state. */
int mfa_profiles_accumulate(mfa_ctx* ctx);

/* ---- fused step ------------------------------------------------------------------------
 * Runs nsteps complete md_main steps (positions, lists, all forces, velocities, energies every
 * energy_every steps, profiles) on the device; graph-captured when opt.use_graphs.
 * Each call first looks, without waiting, at the status words that the previous call copied to
 * the host (once that copy has arrived): a list count past 85 % of the capacity raises the
 * capacity before the new steps.  If the lists of an earlier rebuild overflowed, the capacity is
 * raised, the lists are rebuilt and the call returns MFA_ERR_NLIST_OVERFLOW without running steps
 * (the steps since that rebuild ran on truncated lists); a later call continues normally.     */
int mfa_step(mfa_ctx* ctx, int32_t nsteps);
/* Neighbour-list capacity (entries per particle) and the largest count seen at the rebuilds so
   far.  When the largest count passes 85 % of the capacity, the next mfa_step or
   mfa_verlet_positions raises the capacity by half (up to its maximum) and rebuilds the lists;
   the overflow status of the old capacity is cleared by that rebuild.                         */
int mfa_list_stats(mfa_ctx* ctx, int32_t* capacity, int32_t* max_count);
/* The options the context runs with: those given to mfa_init / mfa_batch_init, with list_cells
   resolved to the value in use.                                                               */
int mfa_get_options(mfa_ctx* ctx, mfa_options* out);
/* Size of the reciprocal-space sum of replica 0: k-vectors of the reference's k-set
   (ewald_k.f90:47-124) and charged particles; both 0 for an uncharged context.  Each replica of a
   charged batch has its own k-set, built from its own box.                                    */
int mfa_kspace_info(mfa_ctx* ctx, int32_t* n_k, int32_t* n_charged);
/* The same for replica rep of a batch (0 <= rep < n_rep; MFA_ERR_ARG otherwise). */
int mfa_kspace_info_replica(mfa_ctx* ctx, int32_t rep, int32_t* n_k, int32_t* n_charged);
/* Absolute step counter of replica 0 (s_time + steps done). */
int mfa_get_step(mfa_ctx* ctx, int64_t* step);

/* ---- data movement --------------------------------------------------------------------- */
/* Any pointer may be NULL. Arrays are 3*n_total doubles in the caller's particle order. */
int mfa_sync_to_host(mfa_ctx* ctx, double* r0, double* v, double* a, double* force);
int mfa_set_state(mfa_ctx* ctx, const double* r0, const double* v, const double* a);
/* Energies of the last energy record, one mfa_energies per replica. */
int mfa_get_energies(mfa_ctx* ctx, mfa_energies* out);
/* Virial and pressure tensors of the last energy record, one mfa_virial per replica: the forces
   and velocities of the record's step (mfa_step every energy_every steps), or the per-routine
   calls since the last mfa_verlet_velocities (each call replaces its own group).               */
int mfa_get_virial(mfa_ctx* ctx, mfa_virial* out);
/* Observation averages of every replica (one mfa_averages each); needs options.observe.        */
int mfa_get_averages(mfa_ctx* ctx, mfa_averages* out);
int mfa_reset_averages(mfa_ctx* ctx);
/* The energy records that mfa_step stored since the previous call (the fort.60/61 series every
   energy_every steps, verlet_velocities.f90:184-207), oldest first: out[k * n_rep + r] is record
   k of replica r, at most cap records; *n = records returned.  Needs options.series_capacity;
   records that the ring overwrote before they were read are lost.                             */
int mfa_get_energy_series(mfa_ctx* ctx, mfa_energies* out, int32_t cap, int32_t* n);
/* Observation quantities of every replica (one mfa_observables each) on the current state; the
   head forces are those of the last energy record (mfa_step every energy_every steps, or the
   last mfa_verlet_velocities call).                                                           */
int mfa_observe(mfa_ctx* ctx, mfa_observables* out);
/* Accumulated profiles of replica rep: dens[hist_dim*3], vsum[hist_dim*3*3], v2sum[...],
   layout [bin][species][dim]; species 0 brush, 1 melt, 2 particle 4.  *n_obs = steps summed. */
int mfa_get_profiles(mfa_ctx* ctx, int32_t rep, double* dens, double* vsum, double* v2sum,
                     int64_t* n_obs);
int mfa_reset_profiles(mfa_ctx* ctx);

/* ---- parity exports -------------------------------------------------------------------- */
/* make_binning + get_cell + neigh_list (cell_list.f90:129-213,56-106) on the device with the
   reference's own grid: cell_of[i] (1-based cell of mobile particle i of replica rep, caller's
   order) and counts[0..n_cells_tot] (counts[0] is the phantom cell); n_cells[3] out.        */
int mfa_cell_list(mfa_ctx* ctx, int32_t rep, int32_t l_box, int32_t* cell_of, int32_t* counts,
                  int32_t counts_cap, int32_t* n_cells);
/* make_cell_list2 (cell_list.f90:285-433) on the device: out[(c-1)*n_nei + k] = k-th
   half-shell neighbour of cell c (0 = phantom), n_nei = 13 (l_box 1) or 62 (l_box 2).        */
int mfa_cell_neigh_list(const int32_t* n_cells, int32_t n_nei, int32_t* out);
/* All interacting pairs (r^2 < range_2, or inside the DPD cut-off where DPD applies) of
   replica rep as 0-based caller-order index pairs i<j; *n = count (may exceed cap).          */
int mfa_pair_list(mfa_ctx* ctx, int32_t rep, int32_t* pairs, int64_t cap, int64_t* n);
/* No counterpart in the reference.  mfa_pair_list that takes no device memory from the
   allocator: for callers that cannot allocate device memory at the point of the call (a host
   program that has handed the device's memory to another component or pool).  The pairs are
   staged in a fixed device array of MFA_PAIR_LIST_STATIC_MAX pairs (2 MiB, held on every device
   that loads the library until exit); cap above that returns MFA_ERR_CAPACITY.  The first call
   on a context looks the array's device address up (make it before any stream capture; a
   context made after a device reset looks it up again).  The call makes the context's device
   current and restores the caller's current device before it returns.  Calls that overlap on
   one device share the array and race.                                                       */
#define MFA_PAIR_LIST_STATIC_MAX 262144
int mfa_pair_list_static(mfa_ctx* ctx, int32_t rep, int32_t* pairs, int64_t cap, int64_t* n);

/* ---- timing ---------------------------------------------------------------------------- */
/* Records CUDA event `slot` (0..15) on the context stream / elapsed ms between two slots. */
int mfa_event_record(mfa_ctx* ctx, int32_t slot);
int mfa_event_elapsed(mfa_ctx* ctx, int32_t slot_a, int32_t slot_b, float* ms);
/* Runs nsteps un-graphed steps with events around each kernel family and returns the mean
   device ms per launch and the launch count per family (names from mfa_kernel_name).  The
   "rebuild" family is the rebuild as mfa_step runs it, per step: the replicas whose skin test
   fired, nothing on most steps; "rebuild_all" is a rebuild of every replica (three, after the
   steps).                                                                                    */
#define MFA_NKFAM 9
int mfa_kernel_times(mfa_ctx* ctx, int32_t nsteps, float* mean_ms, int32_t* launches);
const char* mfa_kernel_name(int32_t fam);
/* FP32 FMA throughput of `device` in TFLOP/s (2 FLOP per FMA), measured by eight independent
   FMA chains per thread on 8 warps per SM sub-partition, best of 10 timed launches: the roof
   for the FP32-issue-bound kernels.  No counterpart in the reference (a measurement aid).    */
int mfa_fp32_fma_peak(int32_t device, double* tflops);
/* Number of kernel launches issued by the library since the context was created. */
int mfa_launch_count(mfa_ctx* ctx, int64_t* n);
/* Number of cell-sort + neighbour-list rebuilds since the context was created (synchronises):
   steps on which some replica was rebuilt. */
int mfa_rebuild_count(mfa_ctx* ctx, int64_t* n);
/* Rebuilds of each replica since the context was created (n_rep counts; synchronises).  The
   decision is per replica: a replica is rebuilt when one of its own particles moved more than
   skin/2 since its last rebuild (check_skin.f90:11-24 decides per system). */
int mfa_replica_rebuild_counts(mfa_ctx* ctx, int64_t* counts);

#ifdef __cplusplus
}
#endif
#endif /* MFA_GPU_H */
