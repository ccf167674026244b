// caviar2_gpu.hpp -- the CAVIAR2 object API on the GB300 MD step.
//
// Same class names, setters and public fields as the reference's API for the
// molecular-dynamics path (inc/caviar2/caviar2.hpp:39-66, domain.hpp:28-133,
// atom_data.hpp:54-720, neighborlist.hpp:34-199, force/lj.hpp:33-150,
// md_simulator.hpp:34-254, tools/atom.hpp, vector3d.hpp:23-39), so that a
// driver such as tests/t001_lj.cpp of the reference builds against it.  The
// objects hold the host mirror of the state in the reference's layouts; the
// step itself runs on the GPU through include/cavgpu.h.  Members are
// initialised (the reference leaves several uninitialised when Caviar2 is
// default-constructed).  Out of scope here: MPI, writers, constraints, molecules.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "cavgpu.h"

namespace caviar2 {

template <typename T>
struct Vector3d {
  Vector3d() : x(0), y(0), z(0) {}
  Vector3d(T x_, T y_, T z_) : x(x_), y(y_), z(z_) {}
  T x, y, z;
};

enum class Integrator_t { Verlet, Velocity_verlet, Leap_frog, Velocity_verlet_langevin, Unknown };

class Caviar2;

class Log {
 public:
  void info(const std::string &s);
  void warning(const std::string &s);
  // prints the message and terminates the process, as the reference (src/log.cpp:190-228)
  [[noreturn]] void error_all(const std::string &s);
};

class Domain {
 public:
  void set_caviar(Caviar2 *c) { caviar_ = c; }
  void set_lower_global(const Vector3d<double> &v) { lower_global = v; }
  void set_upper_global(const Vector3d<double> &v) { upper_global = v; }
  void set_boundary_condition(const Vector3d<int> &v) { boundary_condition = v; }
  void generate();  // single rank: local = global (src/domain.cpp:295-328)
  double volume_global() const { return size_global.x * size_global.y * size_global.z; }

  Vector3d<int> boundary_condition{0, 0, 0};
  Vector3d<double> lower_global, upper_global, lower_local, upper_local, size_local, size_global, half_edge;

 private:
  Caviar2 *caviar_ = nullptr;
};

struct Atom_struct {
  std::vector<size_t> id, type;
  std::vector<Vector3d<double>> position, velocity, acceleration;
};

struct Atom_type_params {
  std::vector<double> mass, mass_inv;
};

namespace tools {
class Atom {
 public:
  explicit Atom(Caviar2 *c = nullptr) : caviar_(c) {}
  void set_type(size_t t) { type = t; }
  void set_position(const Vector3d<double> &p) { position = p; }
  void set_velocity(const Vector3d<double> &v) { velocity = v; }
  size_t type = 0;
  Vector3d<double> position, velocity;

 private:
  Caviar2 *caviar_;
};
}  // namespace tools

class Atom_data {
 public:
  void set_caviar(Caviar2 *c) { caviar_ = c; }
  void set_ghost_cutoff(double v) { ghost_cutoff = v; }
  void set_k_b(double v) { k_b = v; }
  void set_n_r_df(int v) { n_r_df = v; }
  void set_temperature_process(bool v) { temperature_process = v; }
  void set_pressure_process(bool v) { pressure_process = v; }
  void add_type_mass(int type, double m);  // src/atom_data.cpp:368-383
  void add_type_charge(int, double) {}
  // raw add (src/atom_data.cpp:603-637): no domain check
  bool add_atom(size_t id, size_t type, const Vector3d<double> &pos,
                const Vector3d<double> &vel = Vector3d<double>{0.0, 0.0, 0.0});
  // id = current count; rejects atoms outside [lower, upper) (add_unique_atom_molecule.cpp:29-38)
  bool add_atom(tools::Atom &a);
  void reset_owned_acceleration();
  void reset_virial() { virialForce = virialConstraint = virialExternalForce = 0.0; }
  int get_n_r_df();  // src/atom_data.cpp:438-466
  double temperature() const { return temperature_; }
  double pressure() const { return pressure_; }
  double kinetic_energy() const { return kinetic_energy_; }
  double potential_energy() const { return potential_energy_; }  // not in the reference (no PE there)

  Atom_struct atom_struct_owned;
  Atom_type_params atom_type_params;
  double ghost_cutoff = 0.0, k_b = -1.0;
  int n_r_df = -1;
  bool temperature_process = false, pressure_process = false, stochastic_force_present = false;
  double virialForce = 0.0, virialConstraint = 0.0, virialExternalForce = 0.0;

 private:
  friend class Md_simulator;
  friend class force_field_access;
  Caviar2 *caviar_ = nullptr;
  double temperature_ = 0.0, pressure_ = 0.0, kinetic_energy_ = 0.0, potential_energy_ = 0.0;
};

class Neighborlist {
 public:
  void set_caviar(Caviar2 *c) { caviar_ = c; }
  void set_cutoff(double v);
  void set_cutoff_extra_coef(double v);
  void set_make_verlet_list_from_cell_list(bool v) { make_verlet_list_from_cell_list = build_cell_list = v; }
  void set_build_cell_list(bool v) { build_cell_list = v; }
  void set_all_atom_test(bool v) { all_atom_test = v; }
  void set_rebuild_test(bool v) { rebuild_test = v; }
  void set_dt(double v) { dt = v; }

  // The list of the last build in the reference's encoding: neighlist[i] holds owned
  // j > i and, for pairs through a periodic image, N + (index of the image in
  // `ghost_*`).  Filled on request by Md_simulator::export_neighborlist().
  std::vector<std::vector<unsigned int>> neighlist;
  double cutoff = 0.0, cutoff_extra_coef = 1.12347, cutoff_extra = 0.0, dt = 0.0;
  bool make_verlet_list_from_cell_list = false, build_cell_list = false, all_atom_test = false, rebuild_test = false;

 private:
  Caviar2 *caviar_ = nullptr;
};

class Force_field {
 public:
  explicit Force_field(Caviar2 *c) : caviar_(c) {}
  virtual ~Force_field() = default;
  virtual void calculate_acceleration() = 0;
  virtual void verify_settings() {}

 protected:
  Caviar2 *caviar_;
};

namespace force_field {
class Lj : public Force_field {
 public:
  explicit Lj(Caviar2 *c) : Force_field(c) {}
  // Resolves the per-atom (Lorentz-Berthelot), WCA and lambda options into the
  // epsilon / sigma / cutoff_list tables (src/force/lj.cpp:186-381).  As in the
  // reference, nothing calls it on its own: a user of those options calls it.
  void verify_settings() override;
  // The force at the current positions (list rebuilt when the half-skin test
  // asks) into atom_data.atom_struct_owned.acceleration, virial into virialForce.
  void calculate_acceleration() override;
  void set_cutoff(double v);  // throws on negative values (src/force/lj.cpp:74-79)
  void set_epsilon(int t1, int t2, double v);
  void set_sigma(int t1, int t2, double v);
  void set_cutoff_list(const std::vector<std::vector<double>> &v);
  void set_jump_tol(double v);      // enables the jump fix (r^2 floored at v inside the cutoff)
  void enable_wca(bool flag = true);
  void set_lambda_s(const std::vector<std::vector<double>> &v);
  void set_lambda_e(const std::vector<std::vector<double>> &v);
  void set_epsilon_atom(int t, double v);
  void set_sigma_atom(int t, double v);

  double cutoff = 0.0;
  std::vector<std::vector<double>> epsilon, sigma, cutoff_list;
  bool cutoff_list_activated = false;
  bool jump_fix = false, wca = false;
  double jump_tol = 1e-6;
  bool input_by_array = false, input_by_atom = false;
  std::vector<double> epsilon_atom, sigma_atom;
  std::vector<std::vector<double>> lambda_s, lambda_e;
  bool lambda_s_is_set = false, lambda_e_is_set = false;
};
}  // namespace force_field

class Md_simulator {
 public:
  void set_caviar(Caviar2 *c) { caviar_ = c; }
  void set_integrator_type(Integrator_t t);
  void set_initial_step(size_t i) { initial_step = (int64_t)i; use_step = true; }
  void set_final_step(size_t i) { final_step = (int64_t)i; use_step = true; }
  void set_dt(double v) { dt = v; }
  void langevin_temperature(double v);
  void langevin_friction(double v);
  void langevin_kb(double v);
  void langevin_kbt(double v);
  // GPU options (no counterpart in the reference)
  void set_precision(int p) { precision = p; }  // CAVGPU_FP64 (default) or CAVGPU_MIXED
  void set_langevin_seed(uint64_t s) { seed = s; }

  bool run();                 // src/md_simulator.cpp:317-356
  void step();                // src/md_simulator.cpp:445-546
  void step(int64_t i) { current_step = i; step(); }
  void initialize();          // src/md_simulator.cpp:366-420 (creates the GPU context)
  void setup();               // src/md_simulator.cpp:565-611
  void cleanup();             // downloads the state and releases the GPU context
  void sync_host();           // state and thermo of the device copied into the host objects
  void export_neighborlist(); // Neighborlist::neighlist in the reference's encoding
  cavgpu_ctx *gpu_context() { return ctx_; }  // the underlying C-ABI context (after initialize)
  ~Md_simulator();

  double time = 0.0, dt = -1.0;
  int64_t current_step = 0, initial_step = 0, final_step = 0;
  bool use_time = false, use_step = false, initialized = false;
  Integrator_t integrator_type = Integrator_t::Velocity_verlet;
  struct {
    double temperature = -1, friction = 0.0, kb = -1, kbt = -1;
  } langevin_param;
  int precision = CAVGPU_FP64;
  uint64_t seed = 0;
  // ghost images of the last neighborlist export (reference order)
  std::vector<Vector3d<double>> ghost_position;
  std::vector<int32_t> ghost_source;

 private:
  void check(int status, const char *what);
  Caviar2 *caviar_ = nullptr;
  cavgpu_ctx *ctx_ = nullptr;
  bool host_dirty_ = false;
};

class Constraint {
 public:
  explicit Constraint(Caviar2 *c) : caviar_(c) {}
  virtual ~Constraint() = default;

 protected:
  Caviar2 *caviar_;
};

namespace constraint {
// constraint::Nve (inc/caviar2/constraint/nve.hpp, src/constraint/nve.cpp:132-184):
// on steps whose index is a multiple of `step`, velocities are scaled so that the
// kinetic energy is energy_per_dof * dof, energy_tot, dof * kbt / 2 or
// dof * kb * temperature / 2 (the first one set).  Runs on the device, inside the
// step; the GPU path takes at most one Nve, with velocity Verlet or leap-frog.
class Nve : public Constraint {
 public:
  explicit Nve(Caviar2 *c) : Constraint(c) {}
  void verify_settings();  // the reference's checks (src/constraint/nve.cpp:104-130)
  double energy_per_dof = -1.0, energy_tot = -1.0;
  double temperature = -1.0, kb = -1.0, kbt = -1.0;
  int step = 1;
};
}  // namespace constraint

class Caviar2 {
 public:
  Caviar2();
  ~Caviar2() = default;
  Caviar2(const Caviar2 &) = delete;
  Caviar2 &operator=(const Caviar2 &) = delete;

  Atom_data atom_data;
  Domain domain;
  Md_simulator md_simulator;
  Neighborlist neighborlist;
  Log log;
  std::vector<Force_field *> forces;       // non-owning (src/caviar2.cpp:40-44)
  std::vector<Constraint *> constraints;   // non-owning

  void add_force_field(Force_field *f) { forces.push_back(f); }
  void add_constraint(Constraint *c) { constraints.push_back(c); }
};

}  // namespace caviar2
