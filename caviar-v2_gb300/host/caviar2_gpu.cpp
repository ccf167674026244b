// caviar2_gpu.cpp -- CAVIAR2 object API over the cavgpu C ABI (see caviar2_gpu.hpp).
#include "caviar2_gpu.hpp"

#include <algorithm>
#include <charconv>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <deque>
#include <fstream>
#include <mutex>
#include <thread>
#include <unordered_map>

namespace caviar2 {

// ---------------------------------------------------------------- Log
void Log::info(const std::string &s) { std::fprintf(stdout, "[INF] %s\n", s.c_str()); }
void Log::warning(const std::string &s) { std::fprintf(stdout, "[WRN] %s\n", s.c_str()); }
void Log::error_all(const std::string &s) {
  std::fprintf(stderr, "[ERR] %s\n", s.c_str());
  std::fflush(stdout);
  std::exit(1);
}

// ---------------------------------------------------------------- Caviar2
Caviar2::Caviar2() {
  atom_data.set_caviar(this);
  domain.set_caviar(this);
  md_simulator.set_caviar(this);
  neighborlist.set_caviar(this);
}

// ---------------------------------------------------------------- Domain
void Domain::generate() {
  // one rank: grid index 0 of 1 (src/domain.cpp:309-328, 495-502)
  lower_local.x = lower_global.x + (upper_global.x - lower_global.x) * 0 / 1;
  lower_local.y = lower_global.y + (upper_global.y - lower_global.y) * 0 / 1;
  lower_local.z = lower_global.z + (upper_global.z - lower_global.z) * 0 / 1;
  upper_local.x = lower_global.x + (upper_global.x - lower_global.x) * 1 / 1;
  upper_local.y = lower_global.y + (upper_global.y - lower_global.y) * 1 / 1;
  upper_local.z = lower_global.z + (upper_global.z - lower_global.z) * 1 / 1;
  size_local = Vector3d<double>{upper_local.x - lower_local.x, upper_local.y - lower_local.y,
                                upper_local.z - lower_local.z};
  size_global = Vector3d<double>{upper_global.x - lower_global.x, upper_global.y - lower_global.y,
                                 upper_global.z - lower_global.z};
  half_edge = Vector3d<double>{0.5 * size_global.x, 0.5 * size_global.y, 0.5 * size_global.z};
}

// ---------------------------------------------------------------- Atom_data
void Atom_data::add_type_mass(int type, double m) {
  if ((int)atom_type_params.mass.size() < type + 1) {
    atom_type_params.mass.resize(type + 1);
    atom_type_params.mass_inv.resize(type + 1);
  }
  atom_type_params.mass[type] = m;
  atom_type_params.mass_inv[type] = m == 0.0 ? 0.0 : 1.0 / m;
  if (m < 0) caviar_->log.warning("you have entered a negative value for atom mass.");
}

bool Atom_data::add_atom(size_t id, size_t type, const Vector3d<double> &pos, const Vector3d<double> &vel) {
  atom_struct_owned.id.push_back(id);
  atom_struct_owned.type.push_back(type);
  atom_struct_owned.position.push_back(pos);
  atom_struct_owned.velocity.push_back(vel);
  atom_struct_owned.acceleration.push_back(Vector3d<double>{0, 0, 0});
  if (msd_process) atom_struct_owned.msd_domain_cross.push_back(Vector3d<int>{0, 0, 0});
  atom_struct_owned.molecule_index.push_back(-1);
  return true;
}

void Atom_data::zero_msd_domain_cross() {
  auto &m = atom_struct_owned.msd_domain_cross;
  msd_base_.resize(m.size());
  for (size_t j = 0; j < m.size(); ++j) {
    msd_base_[j].x += m[j].x;
    msd_base_[j].y += m[j].y;
    msd_base_[j].z += m[j].z;
    m[j] = Vector3d<int>{0, 0, 0};
  }
}

bool Atom_data::add_atom(tools::Atom &a) {
  const Domain &d = caviar_->domain;
  const auto &p = a.position;
  if (p.x < d.lower_global.x || p.x >= d.upper_global.x || p.y < d.lower_global.y || p.y >= d.upper_global.y ||
      p.z < d.lower_global.z || p.z >= d.upper_global.z)
    return false;
  return add_atom(atom_struct_owned.id.size(), a.type, a.position, a.velocity);
}

void Atom_data::reset_owned_acceleration() {
  for (auto &v : atom_struct_owned.acceleration) v = Vector3d<double>{0, 0, 0};
}

int Atom_data::degree_of_freedoms() { return (int)(3 * atom_struct_owned.position.size()) - get_n_r_df(); }

int Atom_data::get_n_r_df() {
  if (n_r_df == -1) {
    if (stochastic_force_present) {
      n_r_df = 0;
    } else {
      const auto bc = caviar_->domain.boundary_condition;
      const int s = bc.x + bc.y + bc.z;
      n_r_df = s == 0 ? 6 : (s == 3 ? 3 : 6 - s);
    }
  }
  return n_r_df;
}

// ---------------------------------------------------------------- Neighborlist
void Neighborlist::set_cutoff(double v) {
  if (v <= 0.0) caviar_->log.error_all("cutoff have to non-negative.");
  cutoff = v;
}
void Neighborlist::set_cutoff_extra_coef(double v) {
  if (v < 1.0) caviar_->log.error_all("cutoff_extra_coef must be larger than 1.0");
  cutoff_extra_coef = v;
}

// ---------------------------------------------------------------- Lj
namespace force_field {
void Lj::set_cutoff(double v) {
  if (v < 0.0) throw std::runtime_error("Force field cutoff must be non-negative.");
  cutoff = v;
}
void Lj::set_epsilon(int t1, int t2, double v) {
  if ((int)epsilon.size() < t1 + 1) epsilon.resize(t1 + 1);
  if ((int)epsilon[t1].size() < t2 + 1) epsilon[t1].resize(t2 + 1, 0);
  epsilon[t1][t2] = v;
  input_by_array = true;
}
void Lj::set_sigma(int t1, int t2, double v) {
  if ((int)sigma.size() < t1 + 1) sigma.resize(t1 + 1);
  if ((int)sigma[t1].size() < t2 + 1) sigma[t1].resize(t2 + 1, 0);
  sigma[t1][t2] = v;
  input_by_array = true;
}
void Lj::set_jump_tol(double v) {
  jump_fix = true;
  jump_tol = v;
}
void Lj::enable_wca(bool flag) {
  wca = flag;
  if (flag) cutoff_list_activated = true;
}
static void check_non_negative(const std::vector<std::vector<double>> &v, const char *what) {
  for (auto &r : v)
    for (double x : r)
      if (x < 0.0) throw std::runtime_error(std::string(what) + " values must be non-negative.");
}
void Lj::set_lambda_s(const std::vector<std::vector<double>> &v) {
  check_non_negative(v, "Lambda_s");
  lambda_s = v;
  lambda_s_is_set = true;
}
void Lj::set_lambda_e(const std::vector<std::vector<double>> &v) {
  check_non_negative(v, "Lambda_e");
  lambda_e = v;
  lambda_e_is_set = true;
}
void Lj::set_epsilon_atom(int t, double v) {
  if ((int)epsilon_atom.size() < t + 1) epsilon_atom.resize(t + 1, 0);
  epsilon_atom[t] = v;
  input_by_atom = true;
}
void Lj::set_sigma_atom(int t, double v) {
  if ((int)sigma_atom.size() < t + 1) sigma_atom.resize(t + 1, 0);
  sigma_atom[t] = v;
  input_by_atom = true;
}

// The table resolution of the reference's Lj::verify_settings, step by step: the
// tables cover every type present; per-atom input mixes by Lorentz-Berthelot
// (sigma_ij = (sigma_i + sigma_j) / 2, epsilon_ij = sqrt(epsilon_i epsilon_j),
// the diagonal as given); WCA sets cutoff_ij = 2^(1/6) sigma_ij from the mixed
// sigma; lambda_s / lambda_e (missing entries 1) then scale sigma and epsilon.
void Lj::verify_settings() {
  if (input_by_atom && input_by_array) caviar_->log.error_all("lj: (input_by_atom && input_by_array)");
  size_t type_max = 0;
  for (size_t t : caviar_->atom_data.atom_struct_owned.type) type_max = std::max(type_max, t);
  size_t n = 0;
  if (input_by_atom) {
    n = std::max(epsilon_atom.size(), sigma_atom.size());
    epsilon_atom.resize(n, 0);
    sigma_atom.resize(n, 0);
    if (n < type_max + 1) {
      n = type_max + 1;
      epsilon_atom.resize(n, 0);
      sigma_atom.resize(n, 0);
    }
    epsilon.assign(n, std::vector<double>(n, 0));
    sigma.assign(n, std::vector<double>(n, 0));
    for (size_t i = 0; i < n; ++i)
      for (size_t j = 0; j < n; ++j) {
        if (i == j) {
          sigma[i][j] = sigma_atom[i];
          epsilon[i][j] = epsilon_atom[i];
        } else {
          sigma[i][j] = 0.5 * (sigma_atom[i] + sigma_atom[j]);
          epsilon[i][j] = std::sqrt(epsilon_atom[i] * epsilon_atom[j]);
        }
      }
  } else if (input_by_array) {
    n = std::max(epsilon.size(), sigma.size());
    n = std::max(n, type_max + 1);
    epsilon.resize(n);
    sigma.resize(n);
    for (auto &r : epsilon) r.resize(n, 0);
    for (auto &r : sigma) r.resize(n, 0);
  }
  if (wca) {
    const double coef = std::pow(2.0, 1.0 / 6.0);  // the LJ 6-12 minimum
    cutoff_list.assign(n, std::vector<double>(n, 0));
    for (size_t i = 0; i < n; ++i)
      for (size_t j = 0; j < n; ++j) cutoff_list[i][j] = coef * sigma[i][j];
  } else if (cutoff_list_activated) {
    if (cutoff_list.size() < n) cutoff_list.resize(n);
    for (auto &r : cutoff_list)
      if (r.size() < n) r.resize(n, 0);
  }
  auto scale = [&](std::vector<std::vector<double>> &lam, std::vector<std::vector<double>> &tab) {
    if (lam.size() <= type_max) lam.resize(type_max + 1);
    for (auto &r : lam)
      if (r.size() <= type_max) r.resize(type_max + 1, 1.0);
    for (size_t i = 0; i < lam.size() && i < tab.size(); ++i)
      for (size_t j = 0; j < lam[i].size() && j < tab[i].size(); ++j) tab[i][j] *= lam[i][j];
  };
  if (lambda_s_is_set) scale(lambda_s, sigma);
  if (lambda_e_is_set) scale(lambda_e, epsilon);
}
void Lj::set_cutoff_list(const std::vector<std::vector<double>> &v) {
  for (auto &r : v)
    for (double x : r)
      if (x < 0.0) throw std::runtime_error("Cutoff list values must be non-negative.");
  cutoff_list = v;
  cutoff_list_activated = true;
}
void Lj::calculate_acceleration() {
  Md_simulator &md = caviar_->md_simulator;
  if (!md.initialized) {
    md.initialize();
    md.setup();  // computes the force
  } else {
    md.sync_host();
  }
}
}  // namespace force_field

// ---------------------------------------------------------------- constraint::Nve
namespace constraint {
void Nve::verify_settings() {
  const bool kbt_set = kbt > 0.0, temperature_set = temperature > 0.0, kb_set = kb > 0.0;
  if ((temperature_set && kb_set) != (temperature_set || kb_set))
    caviar_->log.error_all("kb and temperature should be set together.");
  const bool t_set = (temperature_set && kb_set) || kbt_set;
  const bool energy_set = energy_per_dof > 0.0 || energy_tot > 0.0;
  if (!(energy_set || t_set)) caviar_->log.error_all("energy or temperature is not set.");
  if (energy_set && t_set) caviar_->log.error_all("Only one of 'energy' and 'temperature' can be set.");
  if (energy_set && energy_per_dof > 0.0 && energy_tot > 0.0)
    caviar_->log.error_all("Only one of 'energy_per_dof' and 'energy_tot' can be set.");
  if (t_set && kbt_set && temperature_set && kb_set)
    caviar_->log.error_all("Only one of 'kbt' and 'temperatue kb' can be set.");
}
}  // namespace constraint

// ---------------------------------------------------------------- Md_simulator
void Md_simulator::check(int status, const char *what) {
  if (status == CAVGPU_OK) return;
  std::string s = std::string(what) + ": " + cavgpu_strerror(status);
  if (status == CAVGPU_E_CUDA) s += std::string(" (") + cavgpu_last_cuda_error() + ")";
  caviar_->log.error_all(s);
}

void Md_simulator::set_integrator_type(Integrator_t t) {
  integrator_type = t;
  if (t == Integrator_t::Unknown) caviar_->log.error_all("invalid or non-implemented integrator");
}
void Md_simulator::langevin_temperature(double v) {
  langevin_param.temperature = v;
  if (v < 0.0) caviar_->log.error_all("Temperature have to non-negative.");
}
void Md_simulator::langevin_friction(double v) {
  langevin_param.friction = v;
  if (v < 0.0) caviar_->log.error_all("friction have to non-negative.");
}
void Md_simulator::langevin_kb(double v) {
  langevin_param.kb = v;
  if (v < 0.0) caviar_->log.error_all("kb have to non-negative.");
}
void Md_simulator::langevin_kbt(double v) {
  langevin_param.kbt = v;
  if (v < 0.0) caviar_->log.error_all("kbt have to non-negative.");
}

Md_simulator::~Md_simulator() {
  if (ctx_) cavgpu_destroy(ctx_);
}

void Md_simulator::initialize() {
  if (dt < 0.0) caviar_->log.error_all("expected 'dt' input");
  if (integrator_type != Integrator_t::Velocity_verlet && integrator_type != Integrator_t::Velocity_verlet_langevin &&
      integrator_type != Integrator_t::Leap_frog)
    caviar_->log.error_all("integrator not on the GPU path (velocity-Verlet, Langevin and leap-frog are)");
  if (caviar_->forces.size() != 1) caviar_->log.error_all("the GPU path runs exactly one force_field::Lj");
  auto *lj = dynamic_cast<force_field::Lj *>(caviar_->forces[0]);
  if (!lj) caviar_->log.error_all("the GPU path runs force_field::Lj");
  Atom_data &ad = caviar_->atom_data;
  Domain &dom = caviar_->domain;
  Neighborlist &nl = caviar_->neighborlist;
  if (ad.k_b < 0) caviar_->log.error_all("k_b is not set.");
  // Atom_data::add_atom(id, type, pos, vel) takes an atom outside the domain, which
  // the reference then treats as another rank's for the whole run (left out of the
  // kinetic energy and temperature); the GPU path takes only atoms inside it, as
  // Atom_data::add_atom(tools::Atom &) does (src/atom_data/add_unique_atom_molecule.cpp:29-38)
  {
    const auto &o = ad.atom_struct_owned;
    for (size_t j = 0; j < o.position.size(); ++j) {
      const auto &x = o.position[j];
      if (x.x < dom.lower_global.x || x.x >= dom.upper_global.x || x.y < dom.lower_global.y ||
          x.y >= dom.upper_global.y || x.z < dom.lower_global.z || x.z >= dom.upper_global.z)
        caviar_->log.error_all("Md_simulator::initialize: the atom with id " + std::to_string(o.id[j]) +
                               " starts outside the domain; the GPU path takes atoms inside it only.");
    }
  }

  cavgpu_params p;
  cavgpu_default_params(&p);
  p.lo[0] = dom.lower_global.x; p.lo[1] = dom.lower_global.y; p.lo[2] = dom.lower_global.z;
  p.hi[0] = dom.upper_global.x; p.hi[1] = dom.upper_global.y; p.hi[2] = dom.upper_global.z;
  p.bc[0] = dom.boundary_condition.x; p.bc[1] = dom.boundary_condition.y; p.bc[2] = dom.boundary_condition.z;
  const int nt = (int)std::max<size_t>(ad.atom_type_params.mass.size(), 1);
  if (nt > CAVGPU_MAX_TYPES) caviar_->log.error_all("too many atom types for the GPU path");
  p.ntypes = nt;
  p.nl_cutoff = nl.cutoff;
  p.nl_coef = nl.cutoff_extra_coef;
  p.lj_cutoff = lj->cutoff;
  for (int a = 0; a < nt; ++a)
    for (int b = 0; b < nt; ++b) {
      // tables as the reference reads them: entries never set are 0 (src/force/lj.cpp:121-140)
      auto at = [](const std::vector<std::vector<double>> &t, int i, int j) {
        return (i < (int)t.size() && j < (int)t[i].size()) ? t[i][j] : 0.0;
      };
      p.eps[a * nt + b] = at(lj->epsilon, a, b);
      p.sigma[a * nt + b] = at(lj->sigma, a, b);
      p.cutoff_list[a * nt + b] = at(lj->cutoff_list, a, b);
    }
  p.cutoff_list_on = lj->cutoff_list_activated ? 1 : 0;
  p.jump_tol = lj->jump_fix ? lj->jump_tol : 0.0;
  for (int t = 0; t < nt; ++t) p.mass[t] = t < (int)ad.atom_type_params.mass.size() ? ad.atom_type_params.mass[t] : 0.0;
  p.k_b = ad.k_b;
  p.dt = dt;
  p.integrator = integrator_type == Integrator_t::Velocity_verlet_langevin ? CAVGPU_VELOCITY_VERLET_LANGEVIN
                 : integrator_type == Integrator_t::Leap_frog              ? CAVGPU_LEAP_FROG
                                                                           : CAVGPU_VELOCITY_VERLET;
  p.lang_temperature = langevin_param.temperature;
  p.lang_friction = langevin_param.friction;
  p.lang_kb = langevin_param.kb;
  p.lang_kbt = langevin_param.kbt;
  p.seed = seed;
  p.n_r_df = ad.get_n_r_df();
  p.pressure_process = ad.pressure_process ? 1 : 0;
  p.precision = precision;
  p.initial_step = initial_step;
  // constraints: the GPU path runs constraint::Nve (at most one)
  int n_nve = 0;
  for (Constraint *cst : caviar_->constraints) {
    auto *nve = dynamic_cast<constraint::Nve *>(cst);
    if (!nve) caviar_->log.error_all("the GPU path runs constraint::Nve only");
    if (++n_nve > 1) caviar_->log.error_all("the GPU path runs one constraint::Nve");
    if (nve->step <= 0) caviar_->log.error_all("Nve: step have to non-negative.");
    p.nve_step = nve->step;
    if (nve->energy_per_dof > 0.0) { p.nve_mode = CAVGPU_NVE_ENERGY_PER_DOF; p.nve_value = nve->energy_per_dof; }
    else if (nve->energy_tot > 0.0) { p.nve_mode = CAVGPU_NVE_ENERGY_TOT; p.nve_value = nve->energy_tot; }
    else if (nve->kbt > 0.0) { p.nve_mode = CAVGPU_NVE_KBT; p.nve_value = nve->kbt; }
    else if (nve->temperature > 0.0 && nve->kb > 0.0) {
      p.nve_mode = CAVGPU_NVE_KB_TEMPERATURE;
      p.nve_value = nve->temperature;
      p.nve_kb = nve->kb;
    } else {
      caviar_->log.error_all("energy or temperature is not set.");
    }
  }
  p.ignore_intra_molecule = lj->ignore_intra_molecule ? 1 : 0;
  p.msd_process = ad.msd_process ? 1 : 0;
  if (ad.msd_process) {  // the device counts from zero: the host mirror keeps its values
    auto &m = ad.atom_struct_owned.msd_domain_cross;
    m.resize(ad.atom_struct_owned.position.size());
    ad.msd_base_.assign(m.size(), Vector3d<int>{0, 0, 0});
    for (size_t j = 0; j < m.size(); ++j) ad.msd_base_[j] = Vector3d<int>{-m[j].x, -m[j].y, -m[j].z};
  }
  if (ctx_) cavgpu_destroy(ctx_);
  ctx_ = nullptr;
  check(cavgpu_create(&p, &ctx_), "cavgpu_create");
  const auto &o = ad.atom_struct_owned;
  static_assert(sizeof(Vector3d<double>) == 3 * sizeof(double), "Vector3d<double> must be three packed doubles");
  static_assert(sizeof(size_t) == sizeof(uint64_t), "size_t must be 64-bit");
  // slot order = insertion order (the noise key is the index, as the reference's
  // per-index draw loop, src/md_simulator.cpp:748-757)
  check(cavgpu_upload(ctx_, (int64_t)o.position.size(), &o.position[0].x, &o.velocity[0].x,
                      reinterpret_cast<const uint64_t *>(o.type.data()), nullptr),
        "cavgpu_upload");
  if (lj->ignore_intra_molecule) {
    std::vector<int32_t> mol(o.position.size(), -1);
    std::copy_n(o.molecule_index.begin(), std::min(mol.size(), o.molecule_index.size()), mol.begin());
    check(cavgpu_set_molecules(ctx_, mol.data()), "cavgpu_set_molecules");
  }
  initialized = true;
}

void Md_simulator::steps_from_time() {
  if (!use_time) return;
  initial_step = (int64_t)((int)initial_time / dt);
  final_step = (int64_t)((int)final_time / dt);
}

void Md_simulator::setup() {
  // setup's time-mode conversion (src/md_simulator.cpp:569-573), then the time of the
  // first step from its index, as Md_simulator::step's first call sets it
  // (src/md_simulator.cpp:458).  The reference sets the time before the conversion,
  // from the index its run() loop then does not use (its run() reads the loop bounds
  // before setup and runs no step in time mode); run() here sets up first and runs
  // from the converted index, so the writers see (step i, time i * dt).
  steps_from_time();
  time = dt * initial_step;
  check(cavgpu_setup(ctx_), "cavgpu_setup");
  // setup takes the temperature, not the pressure (src/md_simulator.cpp:605-607)
  Atom_data &ad = caviar_->atom_data;
  auto &o = ad.atom_struct_owned;
  check(cavgpu_download(ctx_, &o.position[0].x, &o.velocity[0].x, &o.acceleration[0].x), "cavgpu_download");
  read_thermo(false);
  if (ad.msd_process) download_images();
  host_dirty_ = false;
  for (Writer *w : caviar_->writers) w->write(0, 0.0);  // src/md_simulator.cpp:609-610
}

void Md_simulator::autotune(int trial_steps) {
  if (!ctx_) caviar_->log.error_all("autotune: call initialize() and setup() first");
  check(cavgpu_autotune(ctx_, trial_steps, 0, nullptr), "cavgpu_autotune");
}

void Md_simulator::read_thermo(bool with_pressure) {
  Atom_data &ad = caviar_->atom_data;
  double th[6];
  check(cavgpu_thermo(ctx_, th), "cavgpu_thermo");
  ad.kinetic_energy_ = th[0];
  ad.temperature_ = th[1];
  if (with_pressure && ad.pressure_process) ad.pressure_ = th[2];  // finalize_pressure returns early without it
  ad.virialForce = th[3];
  ad.potential_energy_ = th[4];
}

void Md_simulator::download_images() {
  Atom_data &ad = caviar_->atom_data;
  auto &m = ad.atom_struct_owned.msd_domain_cross;
  const size_t n = ad.atom_struct_owned.position.size();
  std::vector<int32_t> img(3 * std::max<size_t>(n, 1));
  check(cavgpu_download_images(ctx_, img.data()), "cavgpu_download_images");
  m.resize(n);
  ad.msd_base_.resize(n);
  for (size_t j = 0; j < n; ++j)
    m[j] = Vector3d<int>{img[3 * j] - ad.msd_base_[j].x, img[3 * j + 1] - ad.msd_base_[j].y,
                         img[3 * j + 2] - ad.msd_base_[j].z};
}

void Md_simulator::sync_host() {
  Atom_data &ad = caviar_->atom_data;
  auto &o = ad.atom_struct_owned;
  check(cavgpu_download(ctx_, &o.position[0].x, &o.velocity[0].x, &o.acceleration[0].x), "cavgpu_download");
  read_thermo(true);
  if (ad.msd_process) download_images();
  host_dirty_ = false;
}

int Md_simulator::writers_want(int64_t i) const {
  int w = 0;
  for (const Writer *wr : caviar_->writers) w |= wr->wants(i);
  return w;
}

void Md_simulator::write_outputs(int64_t i) {
  const int want = writers_want(i);
  if (!want) return;
  Atom_data &ad = caviar_->atom_data;
  const int state = want & (Writer::WANT_POSITIONS | Writer::WANT_VELOCITIES | Writer::WANT_ACCELERATIONS);
  if (state) {  // only the arrays some writer reads
    auto &o = ad.atom_struct_owned;
    check(cavgpu_download(ctx_, (state & Writer::WANT_POSITIONS) ? &o.position[0].x : nullptr,
                          (state & Writer::WANT_VELOCITIES) ? &o.velocity[0].x : nullptr,
                          (state & Writer::WANT_ACCELERATIONS) ? &o.acceleration[0].x : nullptr),
          "cavgpu_download");
    if (state == (Writer::WANT_POSITIONS | Writer::WANT_VELOCITIES | Writer::WANT_ACCELERATIONS)) host_dirty_ = false;
  }
  if ((want & Writer::WANT_CROSSINGS) && ad.msd_process) download_images();
  for (Writer *w : caviar_->writers)
    if (w->wants(i)) w->write(i, time);
}

void Md_simulator::finish_writers() {
  for (Writer *w : caviar_->writers) w->finish();
}

// one step of the reference's loop body (src/md_simulator.cpp:445-546): the
// integrator, then the writers at (current_step, time), then time += dt
void Md_simulator::step() {
  if (!initialized) {
    initialize();
    setup();
  }
  check(cavgpu_step(ctx_, 1), "cavgpu_step");
  read_thermo(true);
  host_dirty_ = true;  // positions stay on the device until sync_host() / run() / cleanup()
  write_outputs(current_step);
  time += dt;
}

// src/md_simulator.cpp:317-356.  The device runs uninterrupted up to the next
// step some writer reads (CUDA graphs of many steps); the host mirror is
// refreshed only there.
void Md_simulator::verify_settings() {
  if (use_time && use_step) caviar_->log.error_all("simulator md: verify_settings: cannot use both 'time' and 'step'.");
  if (!(use_time || use_step)) caviar_->log.error_all("simulator md: verify_settings: please assign 'time' or 'step' variables.");
}

bool Md_simulator::run() {
  caviar_->log.info("MD started.");
  verify_settings();
  if (!initialized) {
    initialize();
    setup();
  }
  current_step = initial_step;
  while (current_step < final_step) {
    int64_t stop = current_step;
    while (stop < final_step - 1 && !writers_want(stop)) ++stop;
    const int64_t n = stop - current_step + 1;
    check(cavgpu_step(ctx_, n), "cavgpu_step");
    for (int64_t k = 0; k + 1 < n; ++k) time += dt;  // the reference's running sum
    current_step = stop;
    read_thermo(true);
    host_dirty_ = true;
    write_outputs(current_step);
    time += dt;
    ++current_step;
  }
  sync_host();
  finish_writers();
  caviar_->log.info("MD finished.");
  return true;
}

void Md_simulator::cleanup() {
  finish_writers();
  if (!ctx_) return;
  if (host_dirty_) sync_host();
  cavgpu_destroy(ctx_);
  ctx_ = nullptr;
  initialized = false;
}

void Md_simulator::export_neighborlist() {
  if (!ctx_) caviar_->log.error_all("export_neighborlist: no GPU state yet");
  Atom_data &ad = caviar_->atom_data;
  Neighborlist &nl = caviar_->neighborlist;
  const size_t n = ad.atom_struct_owned.position.size();
  const int64_t np = cavgpu_export_pairs(ctx_, nullptr, 0);
  if (np < 0) check((int)np, "cavgpu_export_pairs");
  std::vector<int32_t> rows(5 * (size_t)std::max<int64_t>(np, 1));
  check((int)std::min<int64_t>(0, cavgpu_export_pairs(ctx_, rows.data(), np)), "cavgpu_export_pairs");
  // ghost images in the reference's order, for a ghost cutoff no smaller than the list cutoff
  const double ce = nl.cutoff * nl.cutoff_extra_coef;
  const double gc = std::max(ad.ghost_cutoff, ce);
  const int64_t ng = cavgpu_export_ghosts(ctx_, gc, nullptr, nullptr, nullptr, nullptr, 0);
  if (ng < 0) check((int)ng, "cavgpu_export_ghosts");
  std::vector<int32_t> src(std::max<int64_t>(ng, 1)), sh(3 * (size_t)std::max<int64_t>(ng, 1));
  std::vector<double> gp(3 * (size_t)std::max<int64_t>(ng, 1));
  check((int)std::min<int64_t>(0, cavgpu_export_ghosts(ctx_, gc, src.data(), sh.data(), gp.data(), nullptr, ng)),
        "cavgpu_export_ghosts");
  std::unordered_map<int64_t, uint32_t> ghost_of;
  ghost_source.assign(src.begin(), src.begin() + ng);
  ghost_position.resize(ng);
  for (int64_t g = 0; g < ng; ++g) {
    const int code = (sh[3 * g] + 1) + 3 * (sh[3 * g + 1] + 1) + 9 * (sh[3 * g + 2] + 1);
    ghost_of[(int64_t)src[g] * 27 + code] = (uint32_t)g;
    ghost_position[g] = Vector3d<double>{gp[3 * g], gp[3 * g + 1], gp[3 * g + 2]};
  }
  nl.neighlist.assign(n, {});
  for (int64_t r = 0; r < np; ++r) {
    const int32_t *q = &rows[5 * r];
    const int code = (q[2] + 1) + 3 * (q[3] + 1) + 9 * (q[4] + 1);
    if (code == 13) {
      if (q[1] > q[0]) nl.neighlist[q[0]].push_back((unsigned)q[1]);
    } else {
      auto it = ghost_of.find((int64_t)q[1] * 27 + code);
      if (it == ghost_of.end()) caviar_->log.error_all("export_neighborlist: image pair without a ghost");
      nl.neighlist[q[0]].push_back((unsigned)(n + it->second));
    }
  }
  for (auto &r : nl.neighlist) std::sort(r.begin(), r.end());  // the O(N^2) build's order
  nl.cutoff_extra = ce;
}

// ---------------------------------------------------------------- writers
// std::ostream prints a double with the default flags as printf("%.*g", precision);
// std::to_chars with chars_format::general and a precision is specified as that
// same conversion, without the locale and stream machinery.
void append_general6(std::string &out, double v) {
  char buf[40];
  const auto r = std::to_chars(buf, buf + sizeof(buf), v, std::chars_format::general, 6);
  out.append(buf, r.ptr);
}

namespace {
template <class I>
void append_int(std::string &out, I v) {
  char buf[24];
  const auto r = std::to_chars(buf, buf + sizeof(buf), v);
  out.append(buf, r.ptr);
}
}  // namespace

namespace writer {

struct Atom_writer::Impl {
  std::ofstream xyz, energy, temperature, pressure, msd, volume;

  // an xyz frame: a copy of the host mirror, formatted by the worker thread
  struct Frame {
    std::vector<size_t> type, id;
    std::vector<Vector3d<double>> pos, vel, acc;
  };
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Frame> queue;
  bool busy = false, stop = false;
  std::thread worker;

  ~Impl() {
    {
      std::unique_lock<std::mutex> lk(mu);
      stop = true;
    }
    cv.notify_all();
    if (worker.joinable()) worker.join();
  }

  void push(Frame &&f) {
    std::unique_lock<std::mutex> lk(mu);
    if (!worker.joinable()) worker = std::thread([this] { loop(); });
    cv.wait(lk, [this] { return queue.size() < 2; });  // at most two frames held in memory
    queue.push_back(std::move(f));
    cv.notify_all();
  }

  void drain() {
    std::unique_lock<std::mutex> lk(mu);
    cv.wait(lk, [this] { return queue.empty() && !busy; });
  }

  void loop() {
    for (;;) {
      Frame f;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [this] { return stop || !queue.empty(); });
        if (queue.empty()) return;  // stop, nothing left
        f = std::move(queue.front());
        queue.pop_front();
        busy = true;
      }
      cv.notify_all();
      write_frame(f);
      {
        std::unique_lock<std::mutex> lk(mu);
        busy = false;
      }
      cv.notify_all();
    }
  }

  // rows [a, b) of dump_xyz_serial's text (src/writer/atom_writer/dump_xyz_serial.cpp:49-63);
  // the position offset is {0, 0, 0}, and x + 0.0 turns -0.0 into 0.0 as there
  static void rows(const Frame &f, size_t a, size_t b, std::string &out) {
    out.clear();
    out.reserve((b - a) * (24 + 14 * (3 + 3 * !f.vel.empty() + 3 * !f.acc.empty())));
    for (size_t i = a; i < b; ++i) {
      append_int(out, f.type[i]);
      if (!f.id.empty()) { out.push_back(' '); append_int(out, f.id[i]); }
      out.push_back(' '); append_general6(out, f.pos[i].x + 0.0);
      out.push_back(' '); append_general6(out, f.pos[i].y + 0.0);
      out.push_back(' '); append_general6(out, f.pos[i].z + 0.0);
      if (!f.vel.empty()) {
        out.push_back(' '); append_general6(out, f.vel[i].x);
        out.push_back(' '); append_general6(out, f.vel[i].y);
        out.push_back(' '); append_general6(out, f.vel[i].z);
      }
      if (!f.acc.empty()) {
        out.push_back(' '); append_general6(out, f.acc[i].x);
        out.push_back(' '); append_general6(out, f.acc[i].y);
        out.push_back(' '); append_general6(out, f.acc[i].z);
      }
      out.push_back('\n');
    }
  }

  void write_frame(const Frame &f) {
    const size_t n = f.pos.size();
    std::string head;
    append_int(head, n);
    head += "\nAtom\n";
    xyz.write(head.data(), (std::streamsize)head.size());
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t parts = std::max<size_t>(1, std::min<size_t>(hw, n / 16384));
    std::vector<std::string> text(parts);
    std::vector<std::thread> th;
    for (size_t p = 1; p < parts; ++p) th.emplace_back(rows, std::cref(f), n * p / parts, n * (p + 1) / parts, std::ref(text[p]));
    rows(f, 0, n / parts, text[0]);
    for (auto &t : th) t.join();
    for (const auto &t : text) xyz.write(t.data(), (std::streamsize)t.size());
    xyz.flush();
  }
};

Atom_writer::Atom_writer(Caviar2 *c) : Writer(c), impl_(new Impl) { set_caviar(c); }

Atom_writer::~Atom_writer() {
  delete impl_;  // finishes queued frames, then closes the files
}

void Atom_writer::set_caviar(Caviar2 *c) {
  caviar_ = c;
  atom_data = c ? &c->atom_data : nullptr;
  domain = c ? &c->domain : nullptr;
}

void Atom_writer::set_xyz_ghost_step(int step) {
  xyz_ghost_step = step;
  output_xyz_ghost = step > 0;
  if (output_xyz_ghost) caviar_->log.error_all("writer::Atom_writer: ghost xyz output is not on the GPU path");
}

void Atom_writer::set_povray_step(int step) {
  povray_step = step;
  output_povray = step > 0;
  if (output_povray) caviar_->log.error_all("writer::Atom_writer: povray output is not on the GPU path");
}

void Atom_writer::initialize() {
  initialized = true;
  if (output_msd && !atom_data->get_msd_process())
    caviar_->log.error_all("In order to have 'output_msd' in writer::Atom_data, 'msd_process' must be activated in atom_data::Atom_data");
  Impl &m = *impl_;
  if (output_xyz && !m.xyz.is_open()) m.xyz.open(file_name_xyz + ".xyz");
  if (output_energy && !m.energy.is_open()) m.energy.open(file_name_energy + ".txt");
  if (output_temperature && !m.temperature.is_open()) m.temperature.open(file_name_temperature + ".txt");
  if (output_pressure && !m.pressure.is_open()) m.pressure.open(file_name_pressure + ".txt");
  if (output_msd && !m.msd.is_open()) m.msd.open(file_name_msd + ".txt");
  if (output_volume && !m.volume.is_open()) m.volume.open(file_name_volume + ".txt");
}

int Atom_writer::wants(int64_t i) const {
  int w = 0;
  if (output_xyz && i % xyz_step == 0)
    w |= WANT_CALL | WANT_POSITIONS | (xyz_output_velocity ? WANT_VELOCITIES : 0) |
         (xyz_output_acceleration ? WANT_ACCELERATIONS : 0);
  if (output_energy && i % energy_step == 0) w |= WANT_CALL | WANT_THERMO;
  if (output_temperature && i % temperature_step == 0) w |= WANT_CALL | WANT_THERMO;
  if (output_pressure && i % pressure_step == 0) w |= WANT_CALL | WANT_THERMO;
  if (output_msd && i % msd_step == 0 && i >= msd_initial_step) w |= WANT_CALL | WANT_POSITIONS | WANT_CROSSINGS;
  if (output_volume && i % volume_step == 0) w |= WANT_CALL;
  return w;
}

// Atom_writer::write / write_serial (src/writer/atom_writer.cpp:287-303, 427-466)
void Atom_writer::write(int64_t i, double t) {
  if (!initialized) initialize();
  if (output_xyz && i % xyz_step == 0) dump_xyz_serial(i, t);
  if (output_energy && i % energy_step == 0) dump_energy_serial(i, t);
  if (output_temperature && i % temperature_step == 0) dump_temperature_serial(i, t);
  if (output_pressure && i % pressure_step == 0) dump_pressure_serial(i, t);
  if (output_msd && i % msd_step == 0) dump_msd_serial(i, t);
  if (output_volume && i % volume_step == 0) dump_volume_serial(i, t);
}

void Atom_writer::finish() { impl_->drain(); }

void Atom_writer::close_files() {
  impl_->drain();
  for (std::ofstream *f : {&impl_->xyz, &impl_->energy, &impl_->temperature, &impl_->pressure, &impl_->msd,
                           &impl_->volume})
    if (f->is_open()) f->close();
}

void Atom_writer::dump_xyz_serial(int64_t, double) {
  const Atom_struct &o = atom_data->atom_struct_owned;
  Impl::Frame f;
  f.type = o.type;
  if (xyz_output_id) f.id = o.id;
  f.pos = o.position;
  if (xyz_output_velocity) f.vel = o.velocity;
  if (xyz_output_acceleration) f.acc = o.acceleration;
  impl_->push(std::move(f));
}

namespace {
// "i t value" and a flush (src/writer/atom_writer/dump_energy.cpp)
void write_scalar(std::ofstream &f, int64_t i, double t, double v) {
  std::string s;
  append_int(s, i);
  s.push_back(' ');
  append_general6(s, t);
  s.push_back(' ');
  append_general6(s, v);
  s.push_back('\n');
  f.write(s.data(), (std::streamsize)s.size());
  f.flush();
}
}  // namespace

void Atom_writer::dump_energy_serial(int64_t i, double t) { write_scalar(impl_->energy, i, t, atom_data->kinetic_energy()); }
void Atom_writer::dump_temperature_serial(int64_t i, double t) { write_scalar(impl_->temperature, i, t, atom_data->temperature()); }
void Atom_writer::dump_pressure_serial(int64_t i, double t) { write_scalar(impl_->pressure, i, t, atom_data->pressure()); }
void Atom_writer::dump_volume_serial(int64_t i, double t) { write_scalar(impl_->volume, i, t, domain->volume_global()); }

// Atom_writer::dump_msd_serial (src/writer/atom_writer/dump_msd.cpp:35-101), with its
// conventions kept: dr = initial - current + crossings * L, and the y and z crossing
// totals accumulate the x counts.
void Atom_writer::dump_msd_serial(int64_t i, double t) {
  Atom_struct &o = atom_data->atom_struct_owned;
  const auto &pos = o.position;
  const size_t n = pos.size();
  if (i < msd_initial_step) return;
  std::string s;
  if (i == msd_initial_step) {
    msd_initial_position = pos;
    atom_data->zero_msd_domain_cross();
    append_int(s, i);
    s.push_back(' ');
    append_general6(s, t);
    s += " 0.0\n";
    impl_->msd.write(s.data(), (std::streamsize)s.size());
    return;
  }
  if (n != msd_initial_position.size()) caviar_->log.error_all("  (pos.size != msd_initial_position.size())");
  const auto &L = domain->size_global;
  // chunks of 65536 atoms summed on worker threads, then folded in chunk order (the
  // same sum for any thread count; one chunk is the reference's sequential sum)
  struct Part {
    double sum = 0.0;
    long long cross = 0;
    long long count = 0;
  };
  constexpr size_t CHUNK = 65536;
  const size_t nchunk = std::max<size_t>(1, (n + CHUNK - 1) / CHUNK);
  std::vector<Part> part(nchunk);
  auto run_chunk = [&](size_t ck) {
    Part p;
    for (size_t j = ck * CHUNK, e = std::min(n, (ck + 1) * CHUNK); j < e; ++j) {
      if (msd_type > -1 && o.type[j] != static_cast<unsigned int>(msd_type)) continue;
      const auto &c = o.msd_domain_cross[j];
      double dx = msd_initial_position[j].x - pos[j].x;
      double dy = msd_initial_position[j].y - pos[j].y;
      double dz = msd_initial_position[j].z - pos[j].z;
      dx += c.x * L.x;
      dy += c.y * L.y;
      dz += c.z * L.z;
      p.cross += c.x;  // the reference adds the x count to all three totals
      p.sum += dx * dx + dy * dy + dz * dz;
      ++p.count;
    }
    part[ck] = p;
  };
  const size_t nthread = std::min<size_t>(nchunk, std::max(1u, std::thread::hardware_concurrency()));
  if (nthread <= 1) {
    for (size_t ck = 0; ck < nchunk; ++ck) run_chunk(ck);
  } else {
    std::vector<std::thread> th;
    for (size_t w = 0; w < nthread; ++w)
      th.emplace_back([&, w] {
        for (size_t ck = w; ck < nchunk; ck += nthread) run_chunk(ck);
      });
    for (auto &x : th) x.join();
  }
  double sum_dr_sq = 0.0;
  long long cx = 0, count = 0;
  for (const Part &p : part) {
    sum_dr_sq += p.sum;
    cx += p.cross;
    count += p.count;
  }
  const int cross[3] = {(int)cx, (int)cx, (int)cx};
  const double msd = count > 0 ? sum_dr_sq / count : 0.0;
  append_int(s, i);
  s.push_back(' ');
  append_general6(s, t);
  s.push_back(' ');
  append_general6(s, msd);
  for (int a = 0; a < 3; ++a) { s.push_back(' '); append_int(s, cross[a]); }
  s.push_back(' ');
  append_int(s, cross[0] + cross[1] + cross[2]);
  s.push_back('\n');
  impl_->msd.write(s.data(), (std::streamsize)s.size());
  impl_->msd.flush();
}

}  // namespace writer

}  // namespace caviar2
