// lj_md.cpp -- an LJ-fluid run through the CAVIAR2-shaped C++ API, set up the way
// the reference's demo drivers are (tests/t001_lj.cpp, tests/t002_lj.cpp: Domain,
// Atom_data, Neighborlist, force_field::Lj, writer::Atom_writer, Md_simulator::run),
// on an FCC lattice at density 0.8442 and temperature 1.44 (rc 2.5, skin 0.3,
// dt 0.005, velocity Verlet).  Prints one JSON line with the wall time of run().
//
//   lj_md [--cells C] [--steps K | --time T0 T1] [--xyz X] [--thermo T] [--msd M]
//         [--mixed] [--no-tune] [--out PREFIX]
//   C^3 FCC cells (4 C^3 atoms); K steps, or the steps of the time span [T0, T1)
//   (Md_simulator::set_initial_time / set_final_time); xyz frames every X steps,
//   kinetic energy, temperature and pressure every T steps, MSD every M steps
//   (0 = off).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>

#include "caviar2_gpu.hpp"

using namespace caviar2;

int main(int argc, char **argv) {
  int cells = 64, steps = 2000, xyz = 0, thermo = 0, msd = 0;
  double time0 = -1.0, time1 = -1.0;
  bool mixed = false, tune = true;
  std::string out = "lj_md";
  for (int a = 1; a < argc; ++a) {
    auto val = [&](int &v) {
      if (a + 1 >= argc) { std::fprintf(stderr, "%s needs a value\n", argv[a]); std::exit(2); }
      v = std::atoi(argv[++a]);
    };
    if (!std::strcmp(argv[a], "--cells")) val(cells);
    else if (!std::strcmp(argv[a], "--steps")) val(steps);
    else if (!std::strcmp(argv[a], "--xyz")) val(xyz);
    else if (!std::strcmp(argv[a], "--thermo")) val(thermo);
    else if (!std::strcmp(argv[a], "--msd")) val(msd);
    else if (!std::strcmp(argv[a], "--mixed")) mixed = true;
    else if (!std::strcmp(argv[a], "--no-tune")) tune = false;
    else if (!std::strcmp(argv[a], "--out") && a + 1 < argc) out = argv[++a];
    else if (!std::strcmp(argv[a], "--time") && a + 2 < argc) {
      time0 = std::atof(argv[++a]);
      time1 = std::atof(argv[++a]);
    }
    else { std::fprintf(stderr, "unknown option %s\n", argv[a]); return 2; }
  }
  const double rho = 0.8442, temp = 1.44, rc = 2.5, skin = 0.3, dt = 0.005;
  const double a = std::cbrt(4.0 / rho), L = cells * a;

  Caviar2 caviar;
  caviar.domain.set_lower_global(Vector3d<double>{0.0, 0.0, 0.0});
  caviar.domain.set_upper_global(Vector3d<double>{L, L, L});
  caviar.domain.set_boundary_condition(Vector3d<int>{1, 1, 1});
  caviar.domain.generate();

  Atom_data &ad = caviar.atom_data;
  ad.set_ghost_cutoff(rc + skin);
  ad.add_type_mass(0, 1.0);
  ad.set_k_b(1.0);
  ad.set_n_r_df(3);
  ad.set_temperature_process(true);
  ad.set_pressure_process(true);
  if (msd > 0) ad.set_msd_process(true);
  // FCC sites with a quarter-cell offset; Gaussian velocities, zero momentum, scaled to temp
  const double basis[4][3] = {{0, 0, 0}, {0.5, 0.5, 0}, {0.5, 0, 0.5}, {0, 0.5, 0.5}};
  std::mt19937_64 rng(1002);
  std::normal_distribution<double> gauss(0.0, std::sqrt(temp));
  const size_t n = 4 * (size_t)cells * cells * cells;
  std::vector<Vector3d<double>> vel(n);
  Vector3d<double> vsum;
  for (auto &v : vel) {
    v = Vector3d<double>{gauss(rng), gauss(rng), gauss(rng)};
    vsum.x += v.x; vsum.y += v.y; vsum.z += v.z;
  }
  double ke2 = 0.0;
  for (auto &v : vel) {
    v.x -= vsum.x / n; v.y -= vsum.y / n; v.z -= vsum.z / n;
    ke2 += v.x * v.x + v.y * v.y + v.z * v.z;
  }
  const double scale = std::sqrt(temp * (3.0 * n - 3) / ke2);
  size_t k = 0;
  for (int x = 0; x < cells; ++x)
    for (int y = 0; y < cells; ++y)
      for (int z = 0; z < cells; ++z)
        for (const auto &b : basis) {
          const Vector3d<double> p{(x + b[0] + 0.25) * a, (y + b[1] + 0.25) * a, (z + b[2] + 0.25) * a};
          const Vector3d<double> v{vel[k].x * scale, vel[k].y * scale, vel[k].z * scale};
          ad.add_atom(k++, 0, p, v);
        }

  caviar.neighborlist.set_cutoff(rc);
  caviar.neighborlist.set_cutoff_extra_coef((rc + skin) / rc);
  caviar.neighborlist.set_dt(dt);
  caviar.neighborlist.set_make_verlet_list_from_cell_list(true);

  force_field::Lj lj(&caviar);
  lj.set_cutoff(rc);
  lj.set_epsilon(0, 0, 1.0);
  lj.set_sigma(0, 0, 1.0);
  caviar.add_force_field(&lj);

  writer::Atom_writer w(&caviar);
  w.set_xyz_step(xyz);
  w.set_energy_step(thermo);
  w.set_temperature_step(thermo);
  w.set_pressure_step(thermo);
  w.set_msd_step(msd);
  w.set_file_name_xyz(out + "_xyz");
  w.set_file_name_energy(out + "_energy");
  w.set_file_name_temperature(out + "_temperature");
  w.set_file_name_pressure(out + "_pressure");
  w.set_file_name_msd(out + "_msd");
  if (xyz > 0 || thermo > 0 || msd > 0) caviar.add_writer(&w);

  Md_simulator &md = caviar.md_simulator;
  md.set_integrator_type(Integrator_t::Velocity_verlet);
  md.set_precision(mixed ? CAVGPU_MIXED : CAVGPU_FP64);
  md.set_dt(dt);
  if (time0 >= 0.0) {
    md.set_initial_time(time0);
    md.set_final_time(time1);
  } else {
    md.set_initial_step(0);
    md.set_final_step(steps);
  }
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  md.initialize();
  md.setup();
  steps = (int)(md.final_step - md.initial_step);
  if (tune) md.autotune(10);
  const auto t1 = clk::now();
  md.run();
  const auto t2 = clk::now();
  const double setup_s = std::chrono::duration<double>(t1 - t0).count();
  const double run_s = std::chrono::duration<double>(t2 - t1).count();
  std::printf("{\"atoms\": %zu, \"steps\": %d, \"precision\": \"%s\", \"xyz_every\": %d, \"thermo_every\": %d, "
              "\"msd_every\": %d, \"setup_s\": %.4f, \"run_s\": %.4f, \"atom_steps_per_s\": %.6g, "
              "\"T_end\": %.6g, \"initial_step\": %lld, \"final_step\": %lld, \"current_step\": %lld}\n",
              n, steps, mixed ? "mixed" : "fp64", xyz, thermo, msd, setup_s, run_s, (double)n * steps / run_s,
              ad.temperature(), (long long)md.initial_step, (long long)md.final_step, (long long)md.current_step);
  md.cleanup();
  return 0;
}
