// ref_harness.cpp -- drives the UNMODIFIED caviar-md/caviar-v2 library through
// its public C++ API and dumps what the GPU path must reproduce.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/Makefile (target `ref`) from the
// reference's own sources into oracle/_ref/, run by
// tests/golden/make_golden.py to produce the committed golden fixtures, and
// used as the strongest pin of oracle/cav_oracle.c.  Nothing shipped links it.
//
// Input file (little endian), written by tests/golden/make_golden.py:
//   int32  magic 'CAVH', N, ntypes, nsteps, integrator(0 VV,1 Langevin,2 leap-frog),
//          use_cell_list, n_r_df, pressure_process, cutoff_list_on, pad
//   double lo[3], hi[3], nl_cutoff, nl_coef, ghost_cutoff, lj_cutoff, k_b,
//          dt, lang_T, lang_friction, lang_kb
//   double eps[nt*nt], sigma[nt*nt], cutoff_list[nt*nt], mass[nt]
//   double pos[3N], vel[3N]; int32 type[N]
//   extension block, present per bit of the header's last word (`ext`):
//     bit 0: double jump_tol                      -> Lj::set_jump_tol
//     bit 1: (nothing)                            -> Lj::enable_wca
//     bit 2: double eps_atom[nt], sigma_atom[nt]  -> Lj::set_epsilon_atom / set_sigma_atom
//                                                    (instead of set_epsilon / set_sigma)
//     bit 3: double lambda_s[nt*nt], lambda_e[nt*nt] -> Lj::set_lambda_s / set_lambda_e
//     bit 4: int64 step, int32 mode, int32 pad, double value, kb -> constraint::Nve
//            (mode 0 energy_per_dof, 1 energy_tot, 2 kbt, 3 kb + temperature)
//     bit 5: int64 steps of xyz, energy, temperature, pressure, msd, volume output
//            (0 = off); int32 xyz flags (1 id, 2 velocity, 4 acceleration),
//            msd_type, msd_initial_step, pad -> writer::Atom_writer writing
//            <out.bin>_{xyz.xyz, energy.txt, temperature.txt, pressure.txt,
//            msd.txt, volume.txt}; msd output turns Atom_data::msd_process on
//     bit 6: int32 ignore flag, pad, molecule_index[N] -> Atom_struct::molecule_index
//            and Lj::ignore_intra_molecule_flag
//   Bits 1-3 take effect in Lj::verify_settings (src/force/lj.cpp:186-381), which
//   the library itself never calls; the harness calls it, as a user of these
//   options must, and appends the effective tables to the output.
// Output file: see write_* below (sections in fixed order).
//
// Field pinning.  Caviar2 holds Domain/Atom_data/Md_simulator by value and
// default-constructs them (inc/caviar2/caviar2.hpp:46-51, src/caviar2.cpp:20-28),
// which leaves members without initialisers undefined (the cell-list path
// then divides by a garbage Domain::nprocs_x at src/domain.cpp:320-327).  The
// harness constructs Caviar2 in zeroed memory and pins every such field.
// Lj keeps its effective tables private; this test harness reads them after
// verify_settings, so it sees the reference's headers with private members
// exposed (the member layout GCC gives a class does not depend on access).  The
// standard headers come first so that only the reference's own classes change.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>
#define private public
#include "caviar2/caviar2.hpp"
#include "caviar2/constraint/nve.hpp"
#include "caviar2/force/lj.hpp"
#include "caviar2/writer/atom_writer.hpp"
#undef private

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

using namespace caviar2;

namespace {

template <class T> bool rd(FILE *f, T *p, size_t n) { return fread(p, sizeof(T), n, f) == n; }
template <class T> void wr(FILE *f, const T *p, size_t n) { fwrite(p, sizeof(T), n, f); }

void write_pairs(FILE *f, Caviar2 &c) {
  // canonical set: owned-owned pairs both ways with zero shift, owned-ghost
  // pairs as (i, source id, s) with image = pos_src + s*L
  const auto &nl = c.neighborlist.neighlist;
  const auto &gp = c.atom_data.atom_struct_ghost.position;
  const auto &gid = c.atom_data.atom_struct_ghost.id;
  const auto &pos = c.atom_data.atom_struct_owned.position;
  const int N = (int)nl.size();
  std::vector<int32_t> rows;
  for (int i = 0; i < N; ++i)
    for (auto j : nl[i]) {
      if ((int)j >= N) {
        int g = (int)j - N;
        int src = (int)gid[g];
        int32_t s[3];
        double d[3] = {gp[g].x - pos[src].x, gp[g].y - pos[src].y, gp[g].z - pos[src].z};
        double L[3] = {c.domain.size_global.x, c.domain.size_global.y, c.domain.size_global.z};
        for (int k = 0; k < 3; ++k) s[k] = d[k] > 0.5 * L[k] ? 1 : (d[k] < -0.5 * L[k] ? -1 : 0);
        int32_t r[5] = {i, src, s[0], s[1], s[2]};
        rows.insert(rows.end(), r, r + 5);
      } else {
        int32_t r1[5] = {i, (int32_t)j, 0, 0, 0}, r2[5] = {(int32_t)j, i, 0, 0, 0};
        rows.insert(rows.end(), r1, r1 + 5);
        rows.insert(rows.end(), r2, r2 + 5);
      }
    }
  int64_t np = (int64_t)rows.size() / 5;
  wr(f, &np, 1);
  wr(f, rows.data(), rows.size());
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
    return 2;
  }
  FILE *fi = fopen(argv[1], "rb");
  if (!fi) return 3;
  int32_t h[10];
  double dp[15];
  if (!rd(fi, h, 10) || h[0] != 0x48564143) return 4;
  const int N = h[1], nt = h[2], nsteps = h[3], integ = h[4], cell = h[5], nrdf = h[6],
            pproc = h[7], clon = h[8], ext = h[9];
  if (!rd(fi, dp, 15)) return 5;
  std::vector<double> eps(nt * nt), sig(nt * nt), cl(nt * nt), mass(nt), pos(3 * N), vel(3 * N);
  std::vector<int32_t> type(N);
  if (!rd(fi, eps.data(), eps.size()) || !rd(fi, sig.data(), sig.size()) || !rd(fi, cl.data(), cl.size()) ||
      !rd(fi, mass.data(), mass.size()) || !rd(fi, pos.data(), pos.size()) || !rd(fi, vel.data(), vel.size()) ||
      !rd(fi, type.data(), type.size()))
    return 6;
  double jump_tol = 0.0;
  std::vector<double> eps_atom(nt), sig_atom(nt), lam_s(nt * nt), lam_e(nt * nt);
  if ((ext & 1) && !rd(fi, &jump_tol, 1)) return 8;
  if ((ext & 4) && (!rd(fi, eps_atom.data(), nt) || !rd(fi, sig_atom.data(), nt))) return 8;
  if ((ext & 8) && (!rd(fi, lam_s.data(), lam_s.size()) || !rd(fi, lam_e.data(), lam_e.size()))) return 8;
  int64_t nve_step = 0;
  int32_t nve_mode[2] = {0, 0};
  double nve_vk[2] = {0.0, 0.0};
  if ((ext & 16) && (!rd(fi, &nve_step, 1) || !rd(fi, nve_mode, 2) || !rd(fi, nve_vk, 2))) return 8;
  int64_t wsteps[6] = {0, 0, 0, 0, 0, 0};
  int32_t wopt[4] = {0, -1, 0, 0};
  if ((ext & 32) && (!rd(fi, wsteps, 6) || !rd(fi, wopt, 4))) return 8;
  int32_t intra[2] = {0, 0};
  std::vector<int32_t> mol(N, -1);
  if ((ext & 64) && (!rd(fi, intra, 2) || !rd(fi, mol.data(), mol.size()))) return 8;
  fclose(fi);

  void *mem = calloc(1, sizeof(Caviar2));
  Caviar2 &c = *new (mem) Caviar2();

  // ---- Domain (pinned single-rank grid) ----
  c.domain.nprocs_x = c.domain.nprocs_y = c.domain.nprocs_z = 1;
  c.domain.grid_index_x = c.domain.grid_index_y = c.domain.grid_index_z = 0;
  c.domain.me = 0;
  c.domain.nprocs = 1;
  c.domain.set_lower_global(Vector3d<double>{dp[0], dp[1], dp[2]});
  c.domain.set_upper_global(Vector3d<double>{dp[3], dp[4], dp[5]});
  c.domain.set_boundary_condition(Vector3d<int>{1, 1, 1});
  c.domain.generate();

  // ---- Atom_data ----
  c.atom_data.make_ghost_velocity = false;
  c.atom_data.stochastic_force_present = false;
  c.atom_data.set_n_r_df(nrdf);
  c.atom_data.set_ghost_cutoff(dp[8]);
  c.atom_data.set_k_b(dp[10]);
  c.atom_data.set_temperature_process(true);
  c.atom_data.set_pressure_process(pproc != 0);
  for (int t = 0; t < nt; ++t) c.atom_data.add_type_mass(t, mass[t]);
  if (wsteps[4] > 0) c.atom_data.set_msd_process(true);  // before the atoms: add_atom extends msd_domain_cross
  for (int i = 0; i < N; ++i)
    c.atom_data.add_atom((size_t)i, (size_t)type[i], Vector3d<double>{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]},
                         Vector3d<double>{vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]});

  if (ext & 64) {
    // molecules without bonds, angles or dihedrals (degree_of_freedoms reads
    // molecule_struct_owned[index] for every index >= 0)
    int32_t nmol = 0;
    for (int i = 0; i < N; ++i) nmol = std::max(nmol, mol[i] + 1);
    c.atom_data.molecule_struct_owned.resize((size_t)nmol);
    for (int i = 0; i < N; ++i) c.atom_data.atom_struct_owned.molecule_index[i] = mol[i];
  }

  // ---- Neighborlist ----
  c.neighborlist.set_cutoff(dp[6]);
  c.neighborlist.set_cutoff_extra_coef(dp[7]);
  c.neighborlist.set_dt(dp[11]);
  if (cell) c.neighborlist.set_make_verlet_list_from_cell_list(true);

  // ---- force field ----
  force_field::Lj lj(&c);
  lj.set_cutoff(dp[9]);
  if (ext & 4) {
    for (int a = 0; a < nt; ++a) {
      lj.set_epsilon_atom(a, eps_atom[a]);
      lj.set_sigma_atom(a, sig_atom[a]);
    }
  } else {
    for (int a = 0; a < nt; ++a)
      for (int b = 0; b < nt; ++b) {  // both triangles: verify_settings is never called
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
  c.add_force_field(&lj);
  if (ext & 14) lj.verify_settings();
  constraint::Nve nve(&c);
  if (ext & 16) {
    nve.step = (int)nve_step;
    if (nve_mode[0] == 0) nve.energy_per_dof = nve_vk[0];
    else if (nve_mode[0] == 1) nve.energy_tot = nve_vk[0];
    else if (nve_mode[0] == 2) nve.kbt = nve_vk[0];
    else { nve.temperature = nve_vk[0]; nve.kb = nve_vk[1]; }
    c.add_constraint(&nve);
  }
  // ---- writer ----
  writer::Atom_writer aw(&c);
  if (ext & 32) {
    const std::string base = std::string(argv[2]) + "_";
    aw.domain = &c.domain;  // Atom_writer::set_caviar leaves it null; MSD and volume output read it
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
    c.add_writer(&aw);
  }

  // ---- Md_simulator ----
  c.md_simulator.initialized = false;
  c.md_simulator.use_time = false;
  c.md_simulator.langevin_param.kbt = -1;
  if (integ == 1) {
    c.md_simulator.set_integrator_type(Integrator_t::Velocity_verlet_langevin);
    c.md_simulator.langevin_friction(dp[13]);
    c.md_simulator.langevin_kb(dp[14]);
    c.md_simulator.langevin_temperature(dp[12]);
  } else if (integ == 2) {
    c.md_simulator.set_integrator_type(Integrator_t::Leap_frog);
  } else {
    c.md_simulator.set_integrator_type(Integrator_t::Velocity_verlet);
  }
  c.md_simulator.set_dt(dp[11]);
  c.md_simulator.set_initial_step(0);
  c.md_simulator.set_final_step(nsteps);

  // setup (what step() does on its first call)
  c.md_simulator.initialize();
  c.atom_data.reset_virial();
  c.md_simulator.setup();

  FILE *fo = fopen(argv[2], "wb");
  if (!fo) return 7;
  const auto &ad = c.atom_data;
  int32_t n_out = N, g_out = (int32_t)ad.atom_struct_ghost.position.size();
  wr(fo, &n_out, 1);
  wr(fo, &g_out, 1);
  // section 1: acceleration, thermo after setup
  std::vector<double> buf(3 * N);
  for (int i = 0; i < N; ++i) {
    buf[3 * i] = ad.atom_struct_owned.acceleration[i].x;
    buf[3 * i + 1] = ad.atom_struct_owned.acceleration[i].y;
    buf[3 * i + 2] = ad.atom_struct_owned.acceleration[i].z;
  }
  wr(fo, buf.data(), buf.size());
  double th[3] = {c.atom_data.virialForce, c.atom_data.kinetic_energy(), c.atom_data.temperature()};
  wr(fo, th, 3);
  // section 2: bins (cell-list mode only; zeros otherwise), ghosts
  std::vector<int32_t> ib(3 * N, 0), gb(3 * g_out, 0), gsrc(g_out);
  std::vector<double> gpos(3 * g_out);
  for (int i = 0; i < N; ++i)
    if (cell) {
      auto b = c.neighborlist.binlist_index(ad.atom_struct_owned.position[i]);
      ib[3 * i] = b.x; ib[3 * i + 1] = b.y; ib[3 * i + 2] = b.z;
    }
  for (int g = 0; g < g_out; ++g) {
    const auto &q = ad.atom_struct_ghost.position[g];
    if (cell) {
      auto b = c.neighborlist.binlist_index(q);
      gb[3 * g] = b.x; gb[3 * g + 1] = b.y; gb[3 * g + 2] = b.z;
    }
    gsrc[g] = (int32_t)ad.atom_struct_ghost.id[g];
    gpos[3 * g] = q.x; gpos[3 * g + 1] = q.y; gpos[3 * g + 2] = q.z;
  }
  int32_t nb[3] = {c.neighborlist.no_bins.x, c.neighborlist.no_bins.y, c.neighborlist.no_bins.z};
  if (!cell) nb[0] = nb[1] = nb[2] = 0;
  wr(fo, nb, 3);
  wr(fo, ib.data(), ib.size());
  wr(fo, gsrc.data(), gsrc.size());
  wr(fo, gpos.data(), gpos.size());
  wr(fo, gb.data(), gb.size());
  // section 3: canonical pair set of the setup build
  write_pairs(fo, c);
  // section 4: trajectory
  int32_t ns = nsteps;
  wr(fo, &ns, 1);
  for (int s = 0; s < nsteps; ++s) {
    c.md_simulator.step((int64_t)s);
    double t[3] = {c.atom_data.temperature(), c.atom_data.virialForce, c.atom_data.pressure()};
    wr(fo, t, 3);
  }
  for (int part = 0; part < 3; ++part) {
    const auto &v = part == 0 ? ad.atom_struct_owned.position
                              : (part == 1 ? ad.atom_struct_owned.velocity : ad.atom_struct_owned.acceleration);
    for (int i = 0; i < N; ++i) {
      buf[3 * i] = v[i].x; buf[3 * i + 1] = v[i].y; buf[3 * i + 2] = v[i].z;
    }
    wr(fo, buf.data(), buf.size());
  }
  // section 5 (Lj options only): the effective tables after Lj::verify_settings
  if (ext & 14) {
    std::vector<double> te(nt * nt), ts(nt * nt), tc(nt * nt);
    for (int a = 0; a < nt; ++a)
      for (int b = 0; b < nt; ++b) {
        te[a * nt + b] = lj.epsilon[a][b];
        ts[a * nt + b] = lj.sigma[a][b];
        tc[a * nt + b] = lj.cutoff_list_activated ? lj.cutoff_list[a][b] : 0.0;
      }
    int32_t clo = lj.cutoff_list_activated ? 1 : 0;
    wr(fo, te.data(), te.size());
    wr(fo, ts.data(), ts.size());
    wr(fo, tc.data(), tc.size());
    wr(fo, &clo, 1);
  }
  fclose(fo);
  return 0;
}
