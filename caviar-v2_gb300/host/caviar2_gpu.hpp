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
// default-constructed).  Constraints: Nve.  Writers: writer::Atom_writer.  Out of
// scope here: MPI, other constraints and writers, molecules.
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
  double volume_local() const { return size_local.x * size_local.y * size_local.z; }  // src/domain.cpp:433-436
  // a distance component on a periodic axis shifted once by the box edge when it
  // is beyond half of it (src/domain.cpp:330-398)
  double fix_distance_x(double d) const { return fix_axis(d, boundary_condition.x, half_edge.x); }
  double fix_distance_y(double d) const { return fix_axis(d, boundary_condition.y, half_edge.y); }
  double fix_distance_z(double d) const { return fix_axis(d, boundary_condition.z, half_edge.z); }
  Vector3d<double> fix_distance(const Vector3d<double> &v) const {
    return Vector3d<double>{fix_distance_x(v.x), fix_distance_y(v.y), fix_distance_z(v.z)};
  }

  Vector3d<int> boundary_condition{0, 0, 0};
  Vector3d<double> lower_global, upper_global, lower_local, upper_local, size_local, size_global, half_edge;

 private:
  static double fix_axis(double d, int periodic, double h) {
    if (periodic == 1) {
      if (d > +h) d -= h * 2.0;
      if (d < -h) d += h * 2.0;
    }
    return d;
  }
  Caviar2 *caviar_ = nullptr;
};

struct Atom_struct {
  std::vector<size_t> id, type;
  std::vector<Vector3d<double>> position, velocity, acceleration;
  // periodic-boundary crossings per axis (Atom_data::msd_process), +1 through the upper face
  std::vector<Vector3d<int>> msd_domain_cross;
  // molecule of each atom, -1 when none (read by Lj::ignore_intra_molecule)
  std::vector<int32_t> molecule_index;
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
  // the two overloads of the reference (src/atom_data.cpp:327-330, inc/caviar2/atom_data.hpp:695-700)
  void set_msd_process(int flag) { msd_process = flag != 0; }
  void set_msd_process(bool stat) {
    msd_process = stat;
    atom_struct_owned.msd_domain_cross.resize(atom_struct_owned.position.size());
  }
  bool get_msd_process() const { return msd_process; }
  bool get_temperature_process() const { return temperature_process; }
  bool get_pressure_process() const { return pressure_process; }
  long get_num_of_atoms_local() const { return (long)atom_struct_owned.id.size(); }  // src/atom_data.cpp:480-483
  // one rank: the local count (src/atom_data.cpp:484-497)
  long get_num_of_atoms_global() const { return (long)atom_struct_owned.id.size(); }
  // 3N - n_r_df (src/atom_data/kinetic_energy.cpp:642-673; molecules here carry no
  // bonds, angles or dihedrals, so those terms are zero)
  int degree_of_freedoms();
  // msd_domain_cross of every atom set to zero (the writer's MSD origin); the
  // device keeps counting, the host mirror is counted from here
  void zero_msd_domain_cross();
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
  bool temperature_process = false, pressure_process = false, stochastic_force_present = false, msd_process = false;
  double virialForce = 0.0, virialConstraint = 0.0, virialExternalForce = 0.0;

 private:
  friend class Md_simulator;
  friend class force_field_access;
  Caviar2 *caviar_ = nullptr;
  double temperature_ = 0.0, pressure_ = 0.0, kinetic_energy_ = 0.0, potential_energy_ = 0.0;
  // device crossing counts at the host mirror's zero: msd_domain_cross = device - msd_base_
  std::vector<Vector3d<int>> msd_base_;
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
  // pairs of atoms with equal molecule_index take no force (src/force/lj.cpp:93-96, 446);
  // atoms outside molecules share the index -1, so they exclude one another too
  void ignore_intra_molecule_flag(bool flag = true) { ignore_intra_molecule = flag; }
  bool ignore_intra_molecule = false;

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
  void set_initial_time(double t) { initial_time = t; use_time = true; }
  void set_final_time(double t) { final_time = t; use_time = true; }
  // continue a finished run for i more steps (src/md_simulator.cpp:92-97)
  void set_final_add(size_t i) { final_step += (int64_t)i; initial_step = current_step; }
  void verify_settings();  // time or step, not both (src/md_simulator.cpp:358-364)
  // setup()'s time mode (src/md_simulator.cpp:569-573): step = (int)time / dt, the
  // time truncated to an integer before the division, then truncated again
  void steps_from_time();
  void set_dt(double v) { dt = v; }
  void langevin_temperature(double v);
  void langevin_friction(double v);
  void langevin_kb(double v);
  void langevin_kbt(double v);
  // GPU options (no counterpart in the reference)
  void set_precision(int p) { precision = p; }  // CAVGPU_FP64 (default) or CAVGPU_MIXED
  void set_langevin_seed(uint64_t s) { seed = s; }
  // after setup: time the pair-kernel launch shapes on this system and keep the
  // fastest (cavgpu_autotune; the state is restored afterwards)
  void autotune(int trial_steps = 10);

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
  double initial_time = 0.0, final_time = 0.0;
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
  void read_thermo(bool with_pressure);
  void download_images();
  int writers_want(int64_t i) const;   // union of Writer::wants over the writers
  void write_outputs(int64_t i);       // host mirror refreshed as the writers ask, then Writer::write
  void finish_writers();
  Caviar2 *caviar_ = nullptr;
  cavgpu_ctx *ctx_ = nullptr;
  bool host_dirty_ = false;
};

// Writers (inc/caviar2/writer.hpp).  The GPU path adds Writer::wants(): what a
// writer reads at step i, so that the simulator advances the device without a
// host round trip up to the next step some writer reads.
class Writer {
 public:
  enum : int {
    WANT_CALL = 1, WANT_THERMO = 2, WANT_POSITIONS = 4, WANT_VELOCITIES = 8, WANT_ACCELERATIONS = 16,
    WANT_CROSSINGS = 32, WANT_ALL = 63
  };
  explicit Writer(Caviar2 *c = nullptr) : caviar_(c) {}
  virtual ~Writer() = default;
  virtual void initialize() {}
  virtual void write(int64_t, double) {}  // time step and time
  virtual void start_new_files() {}
  virtual void start_new_files(std::string &) {}
  virtual void open_files() {}
  virtual void close_files() {}
  virtual void generate() {}
  virtual void set_caviar(Caviar2 *c) { caviar_ = c; }
  // 0 when write(i, t) would do nothing, else WANT_* bits; a writer of its own
  // (not overriding this) is called with the whole host mirror at every step
  virtual int wants(int64_t) const { return WANT_ALL; }
  // blocks until output handed to background threads is in its files
  virtual void finish() {}

  bool initialized = false;
  int64_t last_timestep = 0;
  double last_time = 0.0, dt = 0.0;
  int my_mpi_rank = 0, mpi_world_size = 1;

 protected:
  Caviar2 *caviar_;
};

namespace writer {
// writer::Atom_writer (inc/caviar2/writer/atom_writer.hpp, src/writer/atom_writer.cpp,
// src/writer/atom_writer/dump_{xyz_serial,energy,msd}.cpp): xyz frames, kinetic
// energy, temperature, pressure, volume and mean square displacement, each every
// X steps, in the reference's text formats (std::ostream default formatting:
// six significant digits).  xyz frames are copied and formatted on background
// threads while the device keeps stepping.  Single process: the *_mpi_* setters
// are kept and have no effect.  Ghost xyz and povray output are not on the GPU
// path (the setters stop with an error).
class Atom_writer : public Writer {
 public:
  explicit Atom_writer(Caviar2 *c);
  ~Atom_writer() override;
  Atom_writer(const Atom_writer &) = delete;
  Atom_writer &operator=(const Atom_writer &) = delete;

  void set_caviar(Caviar2 *c) override;
  void initialize() override;  // opens the files (src/writer/atom_writer.cpp:100-166)
  void write(int64_t i, double t) override;
  int wants(int64_t i) const override;
  void finish() override;
  void close_files() override;

  void set_xyz_mpi_per_process(bool) {}
  void set_xyz_ghost_mpi_per_process(bool) {}
  void set_energy_mpi_per_process(bool) {}
  void set_temperature_mpi_per_process(bool) {}
  void set_pressure_mpi_per_process(bool) {}
  void set_povray_mpi_per_process(bool) {}
  void set_msd_mpi_per_process(bool) {}
  void set_volume_mpi_per_process(bool) {}
  void set_xyz_mpi_rank0(bool) {}
  void set_xyz_ghost_mpi_rank0(bool) {}
  void set_energy_mpi_rank0(bool) {}
  void set_temperature_mpi_rank0(bool) {}
  void set_pressure_mpi_rank0(bool) {}
  void set_povray_mpi_rank0(bool) {}
  void set_msd_mpi_rank0(bool) {}
  void set_volume_mpi_rank0(bool) {}

  void set_xyz_step(int step) { xyz_step = step; output_xyz = step > 0; }
  void set_xyz_ghost_step(int step);
  void set_povray_step(int step);
  void set_energy_step(int step) { energy_step = step; output_energy = step > 0; }
  void set_temperature_step(int step) { temperature_step = step; output_temperature = step > 0; }
  void set_pressure_step(int step) { pressure_step = step; output_pressure = step > 0; }
  void set_msd_step(int step) { msd_step = step; output_msd = step > 0; }
  void set_msd_initial_step(int step) { msd_initial_step = step; }
  void set_volume_step(int step) { volume_step = step; output_volume = step > 0; }

  void set_file_name_xyz(const std::string &fn) { file_name_xyz = fn; }
  void set_file_name_xyz_ghost(const std::string &fn) { file_name_xyz_ghost = fn; }
  void set_file_name_energy(const std::string &fn) { file_name_energy = fn; }
  void set_file_name_temperature(const std::string &fn) { file_name_temperature = fn; }
  void set_file_name_pressure(const std::string &fn) { file_name_pressure = fn; }
  void set_file_name_povray(const std::string &fn) { file_name_povray = fn; }
  void set_file_name_msd(const std::string &fn) { file_name_msd = fn; }
  void set_file_name_volume(const std::string &fn) { file_name_volume = fn; }

  void set_xyz_output_id(int v) { xyz_output_id = v != 0; }
  void set_xyz_output_velocity(int v) { xyz_output_velocity = v != 0; }
  void set_xyz_output_acceleration(int v) { xyz_output_acceleration = v != 0; }
  void set_msd_type(int v) { msd_type = v; }

  void dump_xyz_serial(int64_t i, double t);
  void dump_energy_serial(int64_t i, double t);
  void dump_temperature_serial(int64_t i, double t);
  void dump_pressure_serial(int64_t i, double t);
  void dump_volume_serial(int64_t i, double t);
  void dump_msd_serial(int64_t i, double t);

  Atom_data *atom_data = nullptr;
  Domain *domain = nullptr;  // the reference leaves it null (MSD and volume output then crash)

  bool output_energy = false, output_temperature = false, output_pressure = false, output_xyz = false,
       output_xyz_ghost = false, output_povray = false, output_msd = false, output_volume = false;
  bool xyz_output_velocity = false, xyz_output_acceleration = false, xyz_output_id = false;
  int64_t energy_step = 100, temperature_step = 100, pressure_step = 100, xyz_step = 100, xyz_ghost_step = 100,
          povray_step = 100, msd_step = 100, volume_step = 100;
  int msd_type = -1;         // atom type of the MSD (-1: every atom)
  int msd_initial_step = 0;  // step whose positions are the MSD origin
  std::string file_name_xyz = "o_xyz", file_name_xyz_ghost = "o_xyz_g", file_name_energy = "o_energy",
              file_name_temperature = "o_temperature", file_name_pressure = "o_pressure",
              file_name_povray = "o_pov", file_name_msd = "o_msd", file_name_volume = "o_volume";
  std::vector<Vector3d<double>> msd_initial_position;

 private:
  struct Impl;  // files and the xyz formatting thread
  Impl *impl_ = nullptr;
};
}  // namespace writer

// Text of a double as std::ostream prints it with the default flags and
// precision 6 (printf "%g" of precision 6), appended to out.
void append_general6(std::string &out, double v);

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
// step where the integrator calls apply_thermostat: after the closing kick (velocity
// Verlet, leap-frog) or on the mid-step velocities (Langevin).  At most one Nve.
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
  std::vector<Writer *> writers;           // non-owning (src/caviar2.cpp:51-54)

  void add_force_field(Force_field *f) { forces.push_back(f); }
  void add_constraint(Constraint *c) { constraints.push_back(c); }
  void add_writer(Writer *w) { writers.push_back(w); }
};

}  // namespace caviar2
