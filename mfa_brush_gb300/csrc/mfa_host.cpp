// mfa_host.cpp -- host side of the drop-in: the input files of mfa_brush and the derived tables.
//
// * mfa_flags_from_header: the cpp macros of control_simulation.h (control_simulation.h:9-105) as
//   run-time flags (the reference selects physics at compile time).
// * mfa_read_system_input / mfa_read_mfa_input: Fortran list-directed READ semantics as used by
//   init_system.f90:21-131 and init_params.f90:143-239: a READ with no items skips one record,
//   a READ of k items takes k whitespace/comma-separated values starting at the next record and
//   continuing onto following records if needed, and discards the rest of the last record.
// * mfa_derive_params: init_params.f90:393-887 (sigma rules, 4*epsilon, cut-off and shift rules,
//   wall parameters, DPD noise amplitude, FENE pre-scaling) including the reference's
//   single-precision literals (2.**(1./6.), 2.2, 0.4, 0.98, pi) so that every table entry matches
//   the Fortran bit for bit.
// * mfa_read_conf_old / mfa_write_conf_new: init_config.f90:109-173 and store_config.f90:14-63.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/mfa_gpu.h"

namespace {

constexpr int MX = MFA_MAX_TYPES;
inline int ix(int i, int j) { return i * MX + j; }

struct ListReader {
  std::vector<std::string> lines;
  size_t pos = 0;
  bool open(const char* path) {
    std::ifstream f(path);
    if (!f) return false;
    std::string l;
    while (std::getline(f, l)) lines.push_back(l);
    return true;
  }
  bool skip() {
    if (pos >= lines.size()) return false;
    ++pos;
    return true;
  }
  static void tokenize(const std::string& l, std::vector<std::string>& out) {
    std::string cur;
    for (char c : l) {
      if (std::isspace((unsigned char)c) || c == ',') {
        if (!cur.empty()) out.push_back(cur), cur.clear();
      } else {
        cur.push_back(c);
      }
    }
    if (!cur.empty()) out.push_back(cur);
  }
  // next k tokens (continuing across records)
  bool items(size_t k, std::vector<std::string>& out) {
    out.clear();
    while (out.size() < k) {
      if (pos >= lines.size()) return false;
      std::vector<std::string> t;
      tokenize(lines[pos++], t);
      for (auto& x : t) {
        if (out.size() < k) out.push_back(x);
      }
    }
    return true;
  }
  static bool num(const std::string& t, double& v) {
    std::string u = t;
    for (auto& c : u)
      if (c == 'd' || c == 'D') c = 'e';
    char* end = nullptr;
    v = std::strtod(u.c_str(), &end);
    return end != u.c_str() && *end == '\0';
  }
  bool reals(std::initializer_list<double*> dst) {
    std::vector<std::string> t;
    if (!items(dst.size(), t)) return false;
    size_t k = 0;
    for (double* d : dst)
      if (!num(t[k++], *d)) return false;
    return true;
  }
  template <typename I>
  bool ints(std::initializer_list<I*> dst) {
    std::vector<std::string> t;
    if (!items(dst.size(), t)) return false;
    size_t k = 0;
    for (I* d : dst) {
      double v;
      if (!num(t[k++], v)) return false;
      *d = (I)v;
    }
    return true;
  }
  // one numeric value followed by an ignored token (e.g. "0.1E+01 friction constant")
  bool real_and_word(double* d) {
    std::vector<std::string> t;
    if (!items(1, t)) return false;
    return num(t[0], *d);
  }
};

}  // namespace

extern "C" {

int mfa_flags_from_header(const char* path, mfa_flags* out) {
  if (!path || !out) return MFA_ERR_ARG;
  std::ifstream f(path);
  if (!f) return MFA_ERR_IO;
  mfa_flags F;
  std::memset(&F, 0, sizeof F);
  F.wall = 2;
  F.solvent = 1;
  F.bin_type = 2;
  F.l_box = 1;
  std::string l;
  bool in_comment = false;
  while (std::getline(f, l)) {
    std::string s = l;
    // strip block comments that start and end on this line or span lines
    std::string clean;
    for (size_t k = 0; k < s.size(); ++k) {
      if (in_comment) {
        if (s.compare(k, 2, "*/") == 0) { in_comment = false; ++k; }
        continue;
      }
      if (s.compare(k, 2, "/*") == 0) { in_comment = true; ++k; continue; }
      clean.push_back(s[k]);
    }
    std::istringstream is(clean);
    std::string d, name, val;
    is >> d;
    if (d != "#define" && d != "#undef") continue;
    is >> name;
    is >> val;
    bool def = d == "#define";
    double v = 1.0;
    bool has_val = false;
    if (def && !val.empty()) {
      char* end = nullptr;
      v = std::strtod(val.c_str(), &end);
      has_val = end != val.c_str();
      if (!has_val) v = 1.0;
    }
    auto I = [&](int32_t& x) { x = def ? (int32_t)v : 0; };
    if (name == "SYSTEM") I(F.system);
    else if (name == "SYMMETRY") I(F.symmetry);
    else if (name == "WALL") { if (def) F.wall = (int32_t)v; }
    else if (name == "SOLVENT") { if (def) F.solvent = (int32_t)v; }
    else if (name == "HYDROPHOBIA") I(F.hydrophobia);
    else if (name == "BRUSH_IN_GOOD_SV") I(F.brush_in_good_sv);
    else if (name == "BENDING") I(F.bending);
    else if (name == "BENDING_MELT") I(F.bending_melt);
    else if (name == "ORIENTATION") I(F.orientation);
    else if (name == "PARTICLE_4") I(F.particle_4);
    else if (name == "THERMOSTAT") I(F.thermostat);
    else if (name == "DPD_WEIGHT") I(F.dpd_weight);
    else if (name == "DPD_CUT_OFF") F.dpd_cut_off = def ? v : 0.0;
    else if (name == "FORCE_SWITCH_ON") I(F.force_switch_on);
    else if (name == "POISEUILLE") I(F.poiseuille);
    else if (name == "PROFILES") I(F.profiles);
    else if (name == "BIN_TYPE") { if (def) F.bin_type = (int32_t)v; }
    else if (name == "L_BOX") { if (def) F.l_box = (int32_t)v; }
    else if (name == "FREE_HEADS") I(F.free_heads);
    else if (name == "SHEARED") I(F.sheared);
  }
  *out = F;
  return MFA_OK;
}

int mfa_read_system_input(const char* path, mfa_inputs* io) {
  if (!path || !io) return MFA_ERR_ARG;
  ListReader r;
  if (!r.open(path)) return MFA_ERR_IO;
  const mfa_flags& F = io->flags;
  for (int k = 0; k < 4; ++k)
    if (!r.skip()) return MFA_ERR_PARSE;
  if (!r.ints<int32_t>({&io->n_mon, &io->n_chain, &io->n_cell_w_x, &io->n_cell_w_y})) return MFA_ERR_PARSE;
  r.skip();
  {
    double md, cd;  // n_mon_d, n_chain_d, drop_cell_x, drop_cell_y, z_skin
    if (!r.reals({&md, &cd, &io->drop_cell_x, &io->drop_cell_y, &io->z_skin})) return MFA_ERR_PARSE;
    io->n_mon_d = (int32_t)md;
    io->n_chain_d = (int32_t)cd;
  }
  if (F.particle_4) {
    r.skip();
    if (!r.ints<int32_t>({&io->n_mon_e, &io->n_chain_e, &io->inter4})) return MFA_ERR_PARSE;
  }
  if (F.solvent == 2 || F.solvent == 3) {
    r.skip();
    if (!F.particle_4) {
      if (!r.reals({&io->delta_sig[0]})) return MFA_ERR_PARSE;
    } else {
      if (!r.reals({&io->delta_sig[0], &io->delta_sig[1], &io->delta_sig[2]})) return MFA_ERR_PARSE;
    }
  }
  if (F.wall == 2 || F.wall == 3) {
    r.skip();
    if (F.particle_4) {
      if (!r.reals({&io->a_w, &io->sigma_w, &io->a_w4, &io->sigma_w4})) return MFA_ERR_PARSE;
    } else {
      if (!r.reals({&io->a_w, &io->sigma_w})) return MFA_ERR_PARSE;
    }
  }
  if (F.system == 2 || F.system == 3) {
    r.skip();
    if (!r.reals({&io->charge[0], &io->charge[1], &io->charge[2], &io->charge[3]})) return MFA_ERR_PARSE;
    r.skip();
    double nk;
    if (!r.reals({&io->alpha_c, &nk})) return MFA_ERR_PARSE;
    io->n_kmax = (int32_t)nk;
  }
  if (F.poiseuille) {
    r.skip();
    if (!r.reals({&io->const_force[0], &io->const_force[1], &io->const_force[2]})) return MFA_ERR_PARSE;
  }
  return MFA_OK;
}

int mfa_read_mfa_input(const char* path, mfa_inputs* io) {
  if (!path || !io) return MFA_ERR_ARG;
  ListReader r;
  if (!r.open(path)) return MFA_ERR_IO;
  const mfa_flags& F = io->flags;
  const int nt = (F.wall == 1 && F.particle_4) ? 5 : 4;
  if (!r.ints<int64_t>({&io->s_time})) return MFA_ERR_PARSE;
  if (!r.ints<int64_t>({&io->n_relax})) return MFA_ERR_PARSE;
  if (!r.ints<int64_t>({&io->n_obser})) return MFA_ERR_PARSE;
  if (!r.ints<int64_t>({&io->n_safe})) return MFA_ERR_PARSE;
  if (!r.reals({&io->dt})) return MFA_ERR_PARSE;
  r.skip();
  r.skip();
  if (!r.reals({&io->temp})) return MFA_ERR_PARSE;
  r.skip();
  r.skip();
  r.skip();
  if (!r.reals({&io->x_space})) return MFA_ERR_PARSE;
  if (!r.reals({&io->y_space})) return MFA_ERR_PARSE;
  if (!r.reals({&io->z_space_wall})) return MFA_ERR_PARSE;
  r.skip();
  for (int i = 0; i < nt; ++i) {
    if (!r.reals({&io->mass_type[i]})) return MFA_ERR_PARSE;
    for (int j = 0; j < nt; ++j)
      if (!r.reals({&io->epsil[ix(i, j)]})) return MFA_ERR_PARSE;
    if (!r.reals({&io->sigma_ii[i]})) return MFA_ERR_PARSE;
    if (!r.real_and_word(&io->friction[i])) return MFA_ERR_PARSE;
  }
  if (!r.real_and_word(&io->k_spring_wall)) return MFA_ERR_PARSE;
  if (F.bending) {
    if (!r.reals({&io->k_bend})) return MFA_ERR_PARSE;
    if (!r.reals({&io->alpha_eq})) return MFA_ERR_PARSE;
  }
  r.skip();
  r.skip();
  if (!r.ints<int64_t>({&io->iseed})) return MFA_ERR_PARSE;
  r.skip();
  if (!r.reals({&io->k_chain})) return MFA_ERR_PARSE;
  if (!r.reals({&io->r_chain})) return MFA_ERR_PARSE;
  for (int k = 0; k < 4; ++k) r.skip();
  if (!r.ints<int32_t>({&io->f_twall[0], &io->f_twall[1], &io->f_twall[2]})) return MFA_ERR_PARSE;
  if (!r.reals({&io->va_spring_twall[0], &io->va_spring_twall[1], &io->va_spring_twall[2]})) return MFA_ERR_PARSE;
  if (!F.sheared) {
    if (!r.reals({&io->k_spring_twall[0], &io->k_spring_twall[1], &io->k_spring_twall[2]})) return MFA_ERR_PARSE;
  }
  return MFA_OK;
}

int mfa_derive_params(const mfa_inputs* in, mfa_params* p, mfa_system* s) {
  if (!in || !p || !s) return MFA_ERR_ARG;
  const mfa_flags& F = in->flags;
  if (F.symmetry != 0 || F.free_heads || F.sheared || (F.wall != 1 && F.wall != 2) ||
      (F.system != 0 && F.system != 2 && F.system != 3) || F.dpd_weight > 1)
    return MFA_ERR_UNSUPPORTED;
  std::memset(p, 0, sizeof *p);
  std::memset(s, 0, sizeof *s);
  p->flags = F;
  const int nt = (F.wall == 1 && F.particle_4) ? 5 : 4;  // mfa_common.f90:46-60
  const int W = nt - 1;                                     // index of type n_type
  p->n_type = nt;
  const double c6 = (double)std::pow(2.0f, 1.0f / 6.0f);   // 2.**(1./6.), default REAL
  const double c22 = (double)2.2f;
  auto sq = [](double x) { return x * x; };
  double sg[MX * MX] = {0}, rg[MX * MX] = {0};
  double mass[MX], fric[MX];
  for (int i = 0; i < MX; ++i) mass[i] = in->mass_type[i], fric[i] = in->friction[i];
  for (int i = 0; i < nt; ++i) sg[ix(i, i)] = in->sigma_ii[i];
  if (F.wall == 1 && !F.particle_4) {  // init_params.f90:175-185
    sg[ix(W, W)] = 1.;
    mass[W] = 1.;
    fric[W] = fric[W - 1];
  }
  // sum rule, then the non-additive overrides (init_params.f90:405-453)
  for (int i = 0; i < nt; ++i)
    for (int j = i + 1; j < nt; ++j) sg[ix(i, j)] = sg[ix(j, i)] = (sg[ix(i, i)] + sg[ix(j, j)]) / 2;
  if (F.solvent <= 1) {
    if (!F.particle_4 && F.wall != 1)
      for (int i = 0; i < nt; ++i) sg[ix(i, W)] = sg[ix(W, i)] = 0.;
  } else {
    for (int a : {1, 0}) sg[ix(a, 2)] = sg[ix(2, a)] = in->delta_sig[0];
    if (F.particle_4) {
      for (int a : {1, 0}) sg[ix(a, 3)] = sg[ix(3, a)] = in->delta_sig[1];
      sg[ix(2, 3)] = sg[ix(3, 2)] = in->delta_sig[2];
    }
  }
  for (int i = 0; i < nt; ++i)
    for (int j = 0; j < nt; ++j) {
      p->sigma[ix(i, j)] = sg[ix(i, j)];
      p->sigma_2[ix(i, j)] = sq(sg[ix(i, j)]);
      p->epsil[ix(i, j)] = 4. * in->epsil[ix(i, j)];
    }
  if (F.wall != 1) p->epsil[ix(0, 0)] = 0.;
  // cut-off rules (init_params.f90:497-725), applied in the reference's order
  auto all = [&](auto fn) {
    for (int i = 0; i < nt; ++i)
      for (int j = 0; j < nt; ++j) rg[ix(i, j)] = fn(i, j);
  };
  all([&](int i, int j) { return sq(c6 * sg[ix(i, j)]); });
  rg[ix(0, W)] = sq(c22 * sg[ix(0, W)]);
  rg[ix(W, 0)] = sq(c22 * sg[ix(W, 0)]);
  if (F.wall == 1) {
    if (F.solvent == 0 || F.solvent == 3) {
      const double v = sq(2. * c6 * sg[ix(1, 1)]);
      all([&](int, int) { return v; });
      rg[ix(0, W)] = rg[ix(W, 0)] = rg[ix(W, W)] = 0.;
    } else {
      for (int i = 0; i < nt - 1; ++i)
        for (int j = 0; j < nt - 1; ++j) rg[ix(i, j)] = sq(c6 * sg[ix(i, j)]);
    }
  } else {
    if (F.solvent == 0) {
      all([&](int i, int j) { return sq(2. * c6 * sg[ix(i, j)]); });
      if (!F.particle_4)
        for (int i = 0; i < nt; ++i) rg[ix(i, W)] = rg[ix(W, i)] = 0.;
    }
    if (F.solvent == 3) all([&](int i, int j) { return sq(2. * c6 * sg[ix(i, j)]); });
    if (F.hydrophobia)
      for (auto pr : {std::make_pair(0, 2), std::make_pair(1, 2), std::make_pair(2, 0), std::make_pair(2, 1)})
        rg[ix(pr.first, pr.second)] = sq(c6 * sg[ix(pr.first, pr.second)]);
    if (F.brush_in_good_sv)
      for (auto pr : {std::make_pair(0, 1), std::make_pair(0, 0), std::make_pair(1, 1), std::make_pair(1, 0)})
        rg[ix(pr.first, pr.second)] = sq(c6 * sg[ix(pr.first, pr.second)]);
  }
  if (F.wall == 2) {  // init_params.f90:592-601
    for (int i = 0; i < nt; ++i) {
      p->sigma_wall[i] = (in->sigma_w + sg[ix(i, i)]) / 2;
      p->a_wall[i] = in->a_w;
    }
    if (F.particle_4) {
      p->sigma_wall[3] = (in->sigma_w4 + sg[ix(3, 3)]) / 2.;
      p->a_wall[3] = in->a_w4;
    }
  }
  if (!F.particle_4) {
    if (F.wall == 2)
      for (int i = 0; i < nt; ++i) rg[ix(i, W)] = rg[ix(W, i)] = 0.;
  } else {
    if (F.wall == 1 && F.solvent == 1)
      for (int i = 0; i < nt; ++i) rg[ix(i, W)] = rg[ix(W, i)] = sq(c6 * sg[ix(i, W)]);
    if (F.wall == 1 && F.solvent == 0)
      for (int i = 0; i < nt; ++i) rg[ix(i, W)] = rg[ix(W, i)] = sq(c22 * sg[ix(i, W)]);
    const int i4 = in->inter4;
    if (i4 >= 1 && i4 <= 4) {
      const double f13 = (i4 == 4) ? 2. * c6 : c6;
      for (int i = 0; i < 3; ++i) {
        rg[ix(i, 3)] = sq(f13 * sg[ix(i, 3)]);
        rg[ix(3, i)] = sq(f13 * sg[ix(3, i)]);
      }
      rg[ix(3, 3)] = (i4 == 1) ? sq(c6 * sg[ix(3, 3)]) : sq(2. * (c6 * sg[ix(3, 3)]));
    }
  }
  if (F.system == 0 || F.system == 1 || F.system == 3) rg[ix(0, 0)] = 0.;
  double rmax2 = 0.;
  for (int i = 0; i < nt; ++i)
    for (int j = 0; j < nt; ++j) {
      const double r2 = rg[ix(i, j)];
      p->range_2[ix(i, j)] = r2;
      p->inv_range_2[ix(i, j)] = (r2 != 0) ? 1. / r2 : 0.;
      if (r2 > 0.0) {
        double x = sq(sg[ix(i, j)]) / r2;
        x = x * x * x;
        p->e_shift[ix(i, j)] = x * (x - 1.);
      }
      rmax2 = std::max(rmax2, r2);
    }
  p->r_cut_max = std::sqrt(rmax2);
  if (F.dpd_cut_off > 0) {
    const double rd = (double)(float)F.dpd_cut_off;  // a default-REAL literal in the header
    p->r_cut_max = std::max(rd, p->r_cut_max);
    p->r_cut_dpd_2 = rd * rd;
  }
  p->skin = (double)0.4f;
  p->dt = in->dt;
  p->temp = in->temp;
  for (int i = 0; i < nt; ++i) p->mass_type[i] = mass[i];
  p->friction1 = fric[0];
  p->sig = std::sqrt(2. * in->temp * fric[0] / in->dt);
  p->a_w = in->a_w;
  p->sigma_w = in->sigma_w;
  p->r_chain_2 = in->r_chain * in->r_chain;
  p->inv_r_chain_2 = 1. / p->r_chain_2;
  p->k_chain = in->k_chain * p->r_chain_2;
  p->k_bend = in->k_bend;
  p->alpha_eq = in->alpha_eq;
  p->k_or = in->k_bend;
  p->alpha_or = 0.;
  p->bend_form = in->bend_form;
  for (int d = 0; d < 3; ++d) p->const_force[d] = in->const_force[d];
  for (int i = 0; i < MX; ++i) p->charge[i] = in->charge[i];
  const double pi = (double)3.1415926536f;
  p->alpha_c = in->alpha_c;
  p->sqrt_alpha = std::sqrt(in->alpha_c);
  p->inv_sqrt_pi = (in->compat & MFA_COMPAT_EWALD_INV_PI) ? 1. / pi : 1. / std::sqrt(pi);
  p->n_kmax = in->n_kmax;
  p->rc_coul_2 = (in->compat & MFA_COMPAT_COUL_IN_LJ) ? 0. : in->rc_coul * in->rc_coul;
  p->compat = in->compat;
  p->hist_dim = in->hist_dim > 0 ? in->hist_dim : 200;
  if (in->va_spring_twall[0] != 0. || in->va_spring_twall[1] != 0. || in->va_spring_twall[2] != 0.) {
    // init_params.f90:899-907: moving walls with the body force is an inconsistency the reference
    // stops on.  With explicit walls the wall sites move too (verlet_positions.f90:214-221), in
    // x and y; a z velocity would move them into the channel, which is not built.
    if (F.poiseuille || (F.wall == 1 && in->va_spring_twall[2] != 0.)) return MFA_ERR_UNSUPPORTED;
    p->va_wall[0] = in->va_spring_twall[0];
    p->va_wall[1] = in->va_spring_twall[1];
  }
  s->boundary[0] = in->x_space * (double)in->n_cell_w_x;
  s->boundary[1] = in->y_space * (double)in->n_cell_w_y;
  s->boundary[2] = in->z_space_wall;
  s->n_mon = in->n_mon;
  s->n_chain = in->n_chain;
  s->n_mon_d = in->n_mon_d;
  s->n_chain_d = in->n_chain_d;
  s->n_mon_e = F.particle_4 ? in->n_mon_e : 0;
  s->n_chain_e = F.particle_4 ? in->n_chain_e : 0;
  s->n_mon_tot = in->n_mon * in->n_chain + in->n_mon_d * in->n_chain_d + s->n_mon_e * s->n_chain_e;
  s->n_part = s->n_mon_tot + (F.wall == 1 ? 4 * in->n_cell_w_x * in->n_cell_w_y : 0);
  s->s_time = in->s_time;
  s->seed = (uint64_t)in->iseed;
  return MFA_OK;
}

int mfa_force_switch_on(mfa_params* p, int64_t n_relax, int64_t n_obser) {
  if (!p) return MFA_ERR_ARG;
  (void)n_obser;
  double maxsig = 0.;
  for (int i = 0; i < p->n_type; ++i)
    for (int j = 0; j < p->n_type; ++j) maxsig = std::max(maxsig, p->sigma[ix(i, j)]);
  const double r = (double)0.9f * maxsig;
  p->r_2_min_init = r * r;
  p->r_2_min_time = ((double)n_relax * p->dt < 40.) ? 40. : (double)n_relax * p->dt;
  return MFA_OK;
}

int mfa_read_conf_old(const char* path, int32_t n_part, int32_t* a_type, double* r0, double* v, double* a) {
  if (!path || n_part <= 0 || !a_type || !r0) return MFA_ERR_ARG;
  std::ifstream f(path);
  if (!f) return MFA_ERR_IO;
  std::string l;
  // record 1: flag; 2: (2i10) n_mon n_chain [n_mon_d n_chain_d]; 3: (2i10) wall cells; 4: (i3) order
  for (int k = 0; k < 4; ++k)
    if (!std::getline(f, l)) return MFA_ERR_PARSE;
  for (int i = 0; i < n_part; ++i) {  // (i3,3f13.7)
    if (!std::getline(f, l)) return MFA_ERR_PARSE;
    if (l.size() < 3) return MFA_ERR_PARSE;
    std::istringstream is(l);
    int t;
    double x, y, z;
    if (!(is >> t >> x >> y >> z)) return MFA_ERR_PARSE;
    a_type[i] = t;
    r0[3 * i] = x; r0[3 * i + 1] = y; r0[3 * i + 2] = z;
  }
  for (double* dst : {v, a}) {
    for (int i = 0; i < n_part; ++i) {  // (3f15.7)
      if (!std::getline(f, l)) return MFA_ERR_PARSE;
      std::istringstream is(l);
      double x, y, z;
      if (!(is >> x >> y >> z)) return MFA_ERR_PARSE;
      if (dst) { dst[3 * i] = x; dst[3 * i + 1] = y; dst[3 * i + 2] = z; }
    }
  }
  return MFA_OK;
}

int mfa_write_conf_new(const char* path, const mfa_inputs* in, int32_t n_part, const int32_t* a_type,
                       const double* r0, const double* v, const double* a) {
  if (!path || !in || n_part <= 0 || !a_type || !r0 || !v || !a) return MFA_ERR_ARG;
  FILE* f = std::fopen(path, "w");
  if (!f) return MFA_ERR_IO;
  std::fprintf(f, "1\n");
  std::fprintf(f, "%10d%10d%10d%10d\n", in->n_mon, in->n_chain, in->n_mon_d, in->n_chain_d);
  std::fprintf(f, "%10d%10d\n", in->n_cell_w_x, in->n_cell_w_y);
  std::fprintf(f, "%3d\n", 2);
  for (int i = 0; i < n_part; ++i)
    std::fprintf(f, "%3d%13.7f%13.7f%13.7f\n", a_type[i], r0[3 * i], r0[3 * i + 1], r0[3 * i + 2]);
  for (int i = 0; i < n_part; ++i) std::fprintf(f, "%15.7f%15.7f%15.7f\n", v[3 * i], v[3 * i + 1], v[3 * i + 2]);
  for (int i = 0; i < n_part; ++i) std::fprintf(f, "%15.7f%15.7f%15.7f\n", a[3 * i], a[3 * i + 1], a[3 * i + 2]);
  if (in->flags.wall == 1) {
    // WALL 1 (store_config.f90:47-52): r_wall_equi of every wall bead.  The wall beads follow the
    // mobile particles and are held fixed here, so their equilibrium positions are their positions.
    const long long n_mob = (long long)in->n_mon * in->n_chain + (long long)in->n_mon_d * in->n_chain_d +
                            (long long)in->n_mon_e * in->n_chain_e;
    if (n_mob > n_part) {
      std::fclose(f);
      return MFA_ERR_ARG;
    }
    for (long long i = n_mob; i < n_part; ++i)
      std::fprintf(f, "%15.7f%15.7f%15.7f\n", r0[3 * i], r0[3 * i + 1], r0[3 * i + 2]);
  }
  // top/bottom wall block (r0_twall, rx_twall(:,1:2), pbc_twall, r0_bwall, pbc_bwall,
  // r0_spring_twall, s_force_grad): all zero with walls that do not move
  for (int k = 0; k < 3; ++k) std::fprintf(f, "%15.7f%15.7f%15.7f\n", 0., 0., 0.);
  std::fprintf(f, "%13d%13d%13d\n", 0, 0, 0);
  std::fprintf(f, "%15.7f%15.7f%15.7f\n", 0., 0., 0.);
  std::fprintf(f, "%13d%13d%13d\n", 0, 0, 0);
  std::fprintf(f, "%15.7f%15.7f%15.7f\n", 0., 0., 0.);
  std::fprintf(f, "%13d%13d%13d\n", 0, 0, 0);
  std::fclose(f);
  return MFA_OK;
}

}  // extern "C"
