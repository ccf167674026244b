// host_harness.cpp -- drives the GPU MD step through the CAVIAR2-shaped C++ API
// (caviar-v2_gb300/host/caviar2_gpu.hpp) with the same set-up code a CAVIAR2
// user writes, reading and writing the file formats of oracle/ref_harness.cpp so
// that tests/test_host_api.py compares it with the fixtures the reference made.
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "caviar2_gpu.hpp"

using namespace caviar2;

template <class T> static bool rd(FILE *f, T *p, size_t n) { return fread(p, sizeof(T), n, f) == n; }
template <class T> static void wr(FILE *f, const T *p, size_t n) { fwrite(p, sizeof(T), n, f); }

// The writers' number text (append_general6) against std::ostream's default
// formatting, on values of every magnitude, sign, rounding tie region and kind.
static int format_check() {
  std::vector<double> v = {0.0, -0.0, 1.0, -1.0, 0.1, 1e-4, 9.99999e-5, 1e-5, 123456.0, 1234567.0, 999999.5,
                           9999995.0, 0.0001234565, 2.5, 1e300, -1e-300, 4.9e-324, 1e16, 5e-7,
                           std::numeric_limits<double>::infinity(), -std::numeric_limits<double>::infinity(),
                           std::numeric_limits<double>::max(), std::numeric_limits<double>::min()};
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> u(-1.0, 1.0), e(-320.0, 308.0);
  for (int k = 0; k < 200000; ++k) v.push_back(u(rng) * std::pow(10.0, e(rng)));
  for (int k = 0; k < 200000; ++k) v.push_back(u(rng) * 1000.0);
  for (int k = 0; k < 20000; ++k) v.push_back(std::round(u(rng) * 2e7) / 8.0);  // exact binary ties
  long bad = 0;
  for (double x : v) {
    std::ostringstream os;
    os << x;
    std::string mine;
    append_general6(mine, x);
    if (mine != os.str()) {
      if (bad < 5) fprintf(stderr, "format mismatch: %s vs %s\n", mine.c_str(), os.str().c_str());
      ++bad;
    }
  }
  printf("%zu values, %ld mismatches\n", v.size(), bad);
  return bad ? 1 : 0;
}

// One invalid setting per call, made through the public setters (no GPU is
// touched).  Returns what the reference does: Log::error_all exits with status 1
// after printing "[ERR] <message>"; a setter that throws std::runtime_error is
// reported here as status 2 with "[EXC] <message>"; 0 = nothing was raised.
static int error_case(const std::string &n) {
  Caviar2 c;
  Md_simulator &md = c.md_simulator;
  try {
    if (n == "nl_cutoff") c.neighborlist.set_cutoff(0.0);
    else if (n == "nl_coef") c.neighborlist.set_cutoff_extra_coef(0.5);
    else if (n == "lj_cutoff") { force_field::Lj lj(&c); lj.set_cutoff(-1.0); }
    else if (n == "lang_temperature") md.langevin_temperature(-1.0);
    else if (n == "lang_friction") md.langevin_friction(-1.0);
    else if (n == "integrator") md.set_integrator_type(Integrator_t::Unknown);
    else if (n == "time_and_step") { md.use_time = true; md.set_final_step(10); md.run(); }
    else if (n == "no_time_no_step") md.run();
    else if (n == "nve_kb_alone") { constraint::Nve v(&c); v.kb = 1.0; v.temperature = -1.0; v.verify_settings(); }
    else if (n == "nve_unset") { constraint::Nve v(&c); v.verify_settings(); }
    else if (n == "nve_energy_and_kbt") { constraint::Nve v(&c); v.energy_tot = 1.0; v.kbt = 1.0; v.verify_settings(); }
    else if (n == "outside_start") {  // an atom placed outside the domain before the run (no GPU is reached)
      c.domain.set_lower_global(Vector3d<double>{0.0, 0.0, 0.0});
      c.domain.set_upper_global(Vector3d<double>{6.0, 6.0, 6.0});
      c.domain.set_boundary_condition(Vector3d<int>{1, 1, 1});
      c.atom_data.add_type_mass(0, 1.0);
      c.atom_data.set_k_b(1.0);
      c.atom_data.add_atom((size_t)0, 0, Vector3d<double>{1.0, 1.0, 1.0});
      c.atom_data.add_atom((size_t)1, 0, Vector3d<double>{3.0, 4.0, 6.2});
      force_field::Lj lj(&c);
      c.add_force_field(&lj);
      md.set_dt(0.001);
      md.set_integrator_type(Integrator_t::Velocity_verlet);
      md.initialize();
    }
    else if (n == "valid") { c.neighborlist.set_cutoff(2.5); c.neighborlist.set_cutoff_extra_coef(1.1); }
    else { fprintf(stderr, "unknown error case %s\n", n.c_str()); return 3; }
  } catch (const std::runtime_error &e) {
    fprintf(stderr, "[EXC] %s\n", e.what());
    return 2;
  }
  return 0;
}

int main(int argc, char **argv) {
  if (argc == 2 && !std::strcmp(argv[1], "--format")) return format_check();
  if (argc == 3 && !std::strcmp(argv[1], "--error")) return error_case(argv[2]);
  if (argc == 3 && !std::strcmp(argv[1], "--fix-distance")) {  // box [0,10)x[0,4)x[0,6), periodic x and z
    Caviar2 c;
    c.domain.set_lower_global(Vector3d<double>{0.0, 0.0, 0.0});
    c.domain.set_upper_global(Vector3d<double>{10.0, 4.0, 6.0});
    c.domain.set_boundary_condition(Vector3d<int>{1, 0, 1});
    c.domain.generate();
    const double d = std::atof(argv[2]);
    const Vector3d<double> v = c.domain.fix_distance(Vector3d<double>{d, d, d});
    printf("%.17g %.17g %.17g %.17g %.17g\n", v.x, v.y, v.z, c.domain.volume_local(), c.domain.volume_global());
    return 0;
  }
  if (argc == 4 && !std::strcmp(argv[1], "--counts")) {  // Atom_data counts and flags for n atoms
    Caviar2 c;
    const int n = std::atoi(argv[2]);
    for (int i = 0; i < n; ++i) c.atom_data.add_atom((size_t)i, 0, Vector3d<double>{0.5 * i, 0.0, 0.0});
    c.atom_data.set_n_r_df(std::atoi(argv[3]));
    c.atom_data.set_pressure_process(true);
    printf("%ld %ld %d %d %d\n", c.atom_data.get_num_of_atoms_local(), c.atom_data.get_num_of_atoms_global(),
           c.atom_data.degree_of_freedoms(), (int)c.atom_data.get_temperature_process(),
           (int)c.atom_data.get_pressure_process());
    return 0;
  }
  if (argc == 5 && !std::strcmp(argv[1], "--final-add")) {  // set_final_add after a run ended at `current`
    Caviar2 c;
    Md_simulator &md = c.md_simulator;
    md.set_final_step((size_t)std::atoll(argv[2]));
    md.current_step = std::atoll(argv[3]);
    md.set_final_add((size_t)std::atoll(argv[4]));
    printf("%lld %lld\n", (long long)md.initial_step, (long long)md.final_step);
    return 0;
  }
  if (argc == 5 && !std::strcmp(argv[1], "--time-steps")) {  // setup()'s time-mode conversion only
    Caviar2 c;
    Md_simulator &md = c.md_simulator;
    md.set_dt(std::atof(argv[4]));
    md.set_initial_time(std::atof(argv[2]));
    md.set_final_time(std::atof(argv[3]));
    md.steps_from_time();
    printf("%lld %lld\n", (long long)md.initial_step, (long long)md.final_step);
    return 0;
  }
  if (argc < 3) {
    fprintf(stderr, "usage: %s in.bin out.bin [mixed|tables|run] | --format | --error <case> | --time-steps t0 t1 dt | --final-add final current add | --counts n n_r_df | --fix-distance d\n", argv[0]);
    return 2;
  }
  FILE *fi = fopen(argv[1], "rb");
  if (!fi) return 3;
  int32_t h[10];
  double dp[15];
  if (!rd(fi, h, 10) || h[0] != 0x48564143 || !rd(fi, dp, 15)) return 4;
  const int N = h[1], nt = h[2], nsteps = h[3], integ = h[4], cell = h[5], nrdf = h[6], pproc = h[7], clon = h[8],
            ext = h[9];
  std::vector<double> eps(nt * nt), sig(nt * nt), cl(nt * nt), mass(nt), pos(3 * N), vel(3 * N);
  std::vector<int32_t> type(N);
  if (!rd(fi, eps.data(), eps.size()) || !rd(fi, sig.data(), sig.size()) || !rd(fi, cl.data(), cl.size()) ||
      !rd(fi, mass.data(), mass.size()) || !rd(fi, pos.data(), pos.size()) || !rd(fi, vel.data(), vel.size()) ||
      !rd(fi, type.data(), type.size()))
    return 5;
  // extension block (oracle/ref_harness.cpp): jump_tol, WCA, per-atom eps/sigma, lambda tables
  double jump_tol = 0.0;
  std::vector<double> eps_atom(nt), sig_atom(nt), lam_s(nt * nt), lam_e(nt * nt);
  if ((ext & 1) && !rd(fi, &jump_tol, 1)) return 5;
  if ((ext & 4) && (!rd(fi, eps_atom.data(), nt) || !rd(fi, sig_atom.data(), nt))) return 5;
  if ((ext & 8) && (!rd(fi, lam_s.data(), lam_s.size()) || !rd(fi, lam_e.data(), lam_e.size()))) return 5;
  int64_t nve_step = 0;
  int32_t nve_mode[2] = {0, 0};
  double nve_vk[2] = {0.0, 0.0};
  if ((ext & 16) && (!rd(fi, &nve_step, 1) || !rd(fi, nve_mode, 2) || !rd(fi, nve_vk, 2))) return 5;
  int64_t wsteps[6] = {0, 0, 0, 0, 0, 0};
  int32_t wopt[4] = {0, -1, 0, 0};
  if ((ext & 32) && (!rd(fi, wsteps, 6) || !rd(fi, wopt, 4))) return 5;
  int32_t intra[2] = {0, 0};
  std::vector<int32_t> mol(N, -1);
  if ((ext & 64) && (!rd(fi, intra, 2) || !rd(fi, mol.data(), mol.size()))) return 5;
  fclose(fi);

  Caviar2 caviar;
  caviar.domain.set_lower_global(Vector3d<double>{dp[0], dp[1], dp[2]});
  caviar.domain.set_upper_global(Vector3d<double>{dp[3], dp[4], dp[5]});
  caviar.domain.set_boundary_condition(Vector3d<int>{1, 1, 1});
  caviar.domain.generate();

  caviar.atom_data.set_ghost_cutoff(dp[8]);
  if (wsteps[4] > 0) caviar.atom_data.set_msd_process(true);
  for (int i = 0; i < N; ++i) {
    tools::Atom a(&caviar);
    a.set_type((size_t)type[i]);
    a.set_position(Vector3d<double>{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]});
    a.set_velocity(Vector3d<double>{vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]});
    if (!caviar.atom_data.add_atom(a)) return 6;  // outside the box
  }
  for (int t = 0; t < nt; ++t) caviar.atom_data.add_type_mass(t, mass[t]);
  if (ext & 64)
    for (int i = 0; i < N; ++i) caviar.atom_data.atom_struct_owned.molecule_index[i] = mol[i];
  caviar.atom_data.set_k_b(dp[10]);
  caviar.atom_data.set_n_r_df(nrdf);
  caviar.atom_data.set_temperature_process(true);
  caviar.atom_data.set_pressure_process(pproc != 0);

  caviar.neighborlist.set_cutoff(dp[6]);
  caviar.neighborlist.set_cutoff_extra_coef(dp[7]);
  caviar.neighborlist.set_dt(dp[11]);
  if (cell) caviar.neighborlist.set_make_verlet_list_from_cell_list(true);

  force_field::Lj lj(&caviar);
  lj.set_cutoff(dp[9]);
  if (ext & 4) {
    for (int a = 0; a < nt; ++a) {
      lj.set_epsilon_atom(a, eps_atom[a]);
      lj.set_sigma_atom(a, sig_atom[a]);
    }
  } else {
    for (int a = 0; a < nt; ++a)
      for (int b = 0; b < nt; ++b) {
        lj.set_epsilon(a, b, eps[a * nt + b]);
        lj.set_sigma(a, b, sig[a * nt + b]);
      }
  }
  if (clon) {
    std::vector<std::vector<double>> cll(nt, std::vector<double>(nt));
    for (int a = 0; a < nt; ++a)
      for (int b = 0; b < nt; ++b) cll[a][b] = cl[a * nt + b];
    lj.set_cutoff_list(cll);
  }
  if (ext & 1) lj.set_jump_tol(jump_tol);
  if (ext & 2) lj.enable_wca(true);
  if (ext & 64) lj.ignore_intra_molecule_flag(intra[0] != 0);
  if (ext & 8) {
    std::vector<std::vector<double>> ls(nt, std::vector<double>(nt)), le(nt, std::vector<double>(nt));
    for (int a = 0; a < nt; ++a)
      for (int b = 0; b < nt; ++b) { ls[a][b] = lam_s[a * nt + b]; le[a][b] = lam_e[a * nt + b]; }
    lj.set_lambda_s(ls);
    lj.set_lambda_e(le);
  }
  caviar.add_force_field(&lj);
  if (ext & 14) lj.verify_settings();
  if (argc > 3 && !std::strcmp(argv[3], "tables")) {  // the resolved pair tables only (no GPU needed)
    FILE *fo = fopen(argv[2], "wb");
    if (!fo) return 7;
    auto at = [](const std::vector<std::vector<double>> &t, int i, int j) {
      return (i < (int)t.size() && j < (int)t[i].size()) ? t[i][j] : 0.0;
    };
    for (auto *t : {&lj.epsilon, &lj.sigma, &lj.cutoff_list})
      for (int a = 0; a < nt; ++a)
        for (int b = 0; b < nt; ++b) {
          const double v = at(*t, a, b);
          wr(fo, &v, 1);
        }
    const int32_t clo = lj.cutoff_list_activated ? 1 : 0;
    wr(fo, &clo, 1);
    fclose(fo);
    return 0;
  }

  constraint::Nve nve(&caviar);
  if (ext & 16) {
    nve.step = (int)nve_step;
    if (nve_mode[0] == 0) nve.energy_per_dof = nve_vk[0];
    else if (nve_mode[0] == 1) nve.energy_tot = nve_vk[0];
    else if (nve_mode[0] == 2) nve.kbt = nve_vk[0];
    else { nve.temperature = nve_vk[0]; nve.kb = nve_vk[1]; }
    nve.verify_settings();
    caviar.add_constraint(&nve);
  }

  // writer::Atom_writer with the reference harness's settings and file names
  writer::Atom_writer aw(&caviar);
  if (ext & 32) {
    const std::string base = std::string(argv[2]) + "_";
    aw.set_xyz_step((int)wsteps[0]);
    aw.set_energy_step((int)wsteps[1]);
    aw.set_temperature_step((int)wsteps[2]);
    aw.set_pressure_step((int)wsteps[3]);
    aw.set_msd_step((int)wsteps[4]);
    aw.set_volume_step((int)wsteps[5]);
    aw.set_xyz_output_id(wopt[0] & 1);
    aw.set_xyz_output_velocity((wopt[0] >> 1) & 1);
    aw.set_xyz_output_acceleration((wopt[0] >> 2) & 1);
    aw.set_msd_type(wopt[1]);
    aw.set_msd_initial_step(wopt[2]);
    aw.set_file_name_xyz(base + "xyz");
    aw.set_file_name_energy(base + "energy");
    aw.set_file_name_temperature(base + "temperature");
    aw.set_file_name_pressure(base + "pressure");
    aw.set_file_name_msd(base + "msd");
    aw.set_file_name_volume(base + "volume");
    caviar.add_writer(&aw);
  }

  Md_simulator &md = caviar.md_simulator;
  if (integ == 1) {
    md.set_integrator_type(Integrator_t::Velocity_verlet_langevin);
    md.langevin_friction(dp[13]);
    md.langevin_kb(dp[14]);
    md.langevin_temperature(dp[12]);
  } else if (integ == 2) {
    md.set_integrator_type(Integrator_t::Leap_frog);
  } else {
    md.set_integrator_type(Integrator_t::Velocity_verlet);
  }
  if (argc > 3 && !std::strcmp(argv[3], "mixed")) md.set_precision(CAVGPU_MIXED);
  md.set_dt(dp[11]);
  md.set_initial_step(0);
  md.set_final_step(nsteps);
  md.initialize();
  md.setup();

  FILE *fo = fopen(argv[2], "wb");
  if (!fo) return 7;
  const auto &o = caviar.atom_data.atom_struct_owned;
  md.export_neighborlist();
  const int32_t g = (int32_t)md.ghost_source.size();
  wr(fo, &N, 1);
  wr(fo, &g, 1);
  wr(fo, &o.acceleration[0].x, 3 * (size_t)N);
  double th[3] = {caviar.atom_data.virialForce, caviar.atom_data.kinetic_energy(), caviar.atom_data.temperature()};
  wr(fo, th, 3);
  int32_t nb[3] = {0, 0, 0};
  std::vector<int32_t> ib(3 * (size_t)N, 0);
  if (cell) cavgpu_export_bins(md.gpu_context(), ib.data(), nb);
  std::vector<int32_t> gb(3 * (size_t)g, 0), gsrc(md.ghost_source.begin(), md.ghost_source.end()), gsh(3 * (size_t)g);
  std::vector<double> gpos(3 * (size_t)g);
  if (g > 0) {
    const double gc = caviar.neighborlist.cutoff_extra > caviar.atom_data.ghost_cutoff ? caviar.neighborlist.cutoff_extra
                                                                                    : caviar.atom_data.ghost_cutoff;
    cavgpu_export_ghosts(md.gpu_context(), gc, gsrc.data(), gsh.data(), gpos.data(), gb.data(), g);
  }
  if (!cell) std::fill(gb.begin(), gb.end(), 0);
  wr(fo, nb, 3);
  wr(fo, ib.data(), ib.size());
  wr(fo, gsrc.data(), gsrc.size());
  wr(fo, gpos.data(), gpos.size());
  wr(fo, gb.data(), gb.size());
  // canonical rows from Neighborlist::neighlist (reference encoding)
  std::vector<int32_t> rows;
  const auto &L = caviar.domain.size_global;
  for (int i = 0; i < N; ++i)
    for (unsigned j : caviar.neighborlist.neighlist[i]) {
      if ((int)j >= N) {
        const int gi = (int)j - N, s = md.ghost_source[gi];
        const auto &q = md.ghost_position[gi];
        const double dd[3] = {q.x - o.position[s].x, q.y - o.position[s].y, q.z - o.position[s].z};
        const double LL[3] = {L.x, L.y, L.z};
        int32_t r[5] = {i, s, 0, 0, 0};
        for (int k = 0; k < 3; ++k) r[2 + k] = dd[k] > 0.5 * LL[k] ? 1 : (dd[k] < -0.5 * LL[k] ? -1 : 0);
        rows.insert(rows.end(), r, r + 5);
      } else {
        int32_t r1[5] = {i, (int32_t)j, 0, 0, 0}, r2[5] = {(int32_t)j, i, 0, 0, 0};
        rows.insert(rows.end(), r1, r1 + 5);
        rows.insert(rows.end(), r2, r2 + 5);
      }
    }
  int64_t np = (int64_t)rows.size() / 5;
  wr(fo, &np, 1);
  wr(fo, rows.data(), rows.size());
  wr(fo, &nsteps, 1);
  if (argc > 3 && !std::strcmp(argv[3], "run")) {
    // Md_simulator::run: the device advances between the steps the writers read;
    // only the last step's thermo exists (written for every record)
    md.run();
    double t[3] = {caviar.atom_data.temperature(), caviar.atom_data.virialForce, caviar.atom_data.pressure()};
    for (int s = 0; s < nsteps; ++s) wr(fo, t, 3);
  } else {
    for (int s = 0; s < nsteps; ++s) {
      md.step((int64_t)s);
      double t[3] = {caviar.atom_data.temperature(), caviar.atom_data.virialForce, caviar.atom_data.pressure()};
      wr(fo, t, 3);
    }
  }
  md.sync_host();
  aw.finish();
  wr(fo, &o.position[0].x, 3 * (size_t)N);
  wr(fo, &o.velocity[0].x, 3 * (size_t)N);
  wr(fo, &o.acceleration[0].x, 3 * (size_t)N);
  fclose(fo);
  md.cleanup();
  return 0;
}
