/*
 * cav_oracle.h -- CPU restatement of CAVIAR2's molecular-dynamics step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle the GPU path is tested
 * against: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * may load it.  The product (libcavgpu.so) never links or calls it.
 *
 * It restates, in plain C, the single-rank CPU path of caviar-md/caviar-v2:
 *   Domain::fix_position               src/domain.cpp:443-493
 *   exchange_ghost_single_md_domain    src/atom_data/exchange_ghost_single_md_domain.cpp:24-215
 *   Neighborlist::init/build/...       src/neighborlist.cpp:77-148, 247-297, 303-672
 *   force_field::Lj::calculate_acceleration  src/force/lj.cpp:393-517
 *   Md_simulator::setup/step/integrate_*     src/md_simulator.cpp:422-869
 *   Atom_data::kinetic_energy/temperature/pressure  src/atom_data/kinetic_energy.cpp:26-303
 * with the same loop orders and floating-point expression orders, so that it
 * reproduces the reference bit for bit when both are built with
 * -ffp-contract=off.  Parity of this restatement is pinned against the
 * reference itself: tests/golden/make_golden.py compiles the reference's own
 * sources (oracle/Makefile, target `ref`) and stores its outputs as fixtures.
 *
 * Two deliberate differences, both named by the GPU design:
 *   - Langevin noise is counter-based Philox4x32-10 keyed by (seed, atom id,
 *     step) instead of three std::mt19937 streams (the reference's streams are
 *     left unseeded by Caviar2's default constructor and give eta_x == eta_y
 *     == eta_z).  noise_mode 0 switches the noise off (eta = 0) for exact
 *     comparison with the reference.
 *   - A potential energy is computed (the reference has none:
 *     src/force_field.cpp:39-43); V(r) is the pair potential whose -dV/dr
 *     equals the reference force (shifted-force LJ).
 */
#ifndef CAV_ORACLE_H
#define CAV_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_TYPES 8

typedef struct orc_params {
  double lo[3], hi[3];          /* Domain::set_lower_global / set_upper_global */
  int32_t bc[3];                /* Domain::set_boundary_condition (1 = periodic) */
  int32_t ntypes;
  double nl_cutoff;             /* Neighborlist::set_cutoff */
  double nl_coef;               /* Neighborlist::set_cutoff_extra_coef */
  double ghost_cutoff;          /* Atom_data::set_ghost_cutoff */
  double lj_cutoff;             /* Lj::set_cutoff */
  double eps[ORC_MAX_TYPES * ORC_MAX_TYPES];      /* Lj::set_epsilon, [ti*ntypes+tj] */
  double sigma[ORC_MAX_TYPES * ORC_MAX_TYPES];    /* Lj::set_sigma */
  double cutoff_list[ORC_MAX_TYPES * ORC_MAX_TYPES]; /* Lj::set_cutoff_list */
  double mass[ORC_MAX_TYPES];   /* Atom_data::add_type_mass */
  double k_b;                   /* Atom_data::set_k_b */
  double dt;                    /* Md_simulator::set_dt */
  double lang_temperature, lang_friction, lang_kb, lang_kbt;
  uint64_t seed;                /* Philox key for Langevin noise */
  int32_t cutoff_list_on;
  int32_t use_cell_list;        /* Neighborlist::set_make_verlet_list_from_cell_list */
  int32_t n_r_df;               /* Atom_data::set_n_r_df (0..3) */
  int32_t integrator;           /* 0 velocity-Verlet, 1 velocity-Verlet-Langevin, 2 leap-frog */
  int32_t noise_mode;           /* Langevin: 0 eta = 0, 1 Philox */
  int32_t pressure_process;     /* Atom_data::set_pressure_process */
  int32_t rebuild_test;         /* Neighborlist::set_rebuild_test: rebuild on every step */
  double jump_tol;              /* Lj::set_jump_tol (src/force/lj.cpp:82-86); 0 = off */
  int64_t nve_step;             /* constraint::Nve every nve_step steps; 0 = off */
  int32_t nve_mode;             /* 0 energy_per_dof, 1 energy_tot, 2 kbt, 3 kb + temperature */
  int32_t ignore_intra;         /* Lj::ignore_intra_molecule_flag (src/force/lj.cpp:93-96, 446) */
  double nve_value, nve_kb;
} orc_params;

typedef struct orc_sys orc_sys;

/* Status codes (negative = error). */
#define ORC_OK 0
#define ORC_E_ARG -1
#define ORC_E_NAN -2
#define ORC_E_NOMEM -3

orc_sys *orc_new(const orc_params *p, int32_t n, const double *pos3,
                 const double *vel3, const int32_t *type);
void orc_free(orc_sys *s);

/* Md_simulator::initialize + setup (src/md_simulator.cpp:366-420, 565-611). */
int32_t orc_setup(orc_sys *s);
/* nsteps calls of Md_simulator::step (src/md_simulator.cpp:445-546). */
int32_t orc_step(orc_sys *s, int32_t nsteps);

/* State and observables. */
void orc_get_state(const orc_sys *s, double *pos3, double *vel3, double *acc3);
/* out[0..5] = KE, T, P, virialForce, PE, rebuild count */
void orc_get_thermo(const orc_sys *s, double *out6);
/* Atom_struct::msd_domain_cross per atom, x3 (crossings since orc_new) */
void orc_get_images(const orc_sys *s, int32_t *img3);
/* Atom_struct::molecule_index per atom (-1 for every atom until set, as add_atom) */
int32_t orc_set_molecules(orc_sys *s, const int32_t *mol);
int64_t orc_current_step(const orc_sys *s);

/* Neighbour list, ghosts and cells of the last build. */
int64_t orc_pair_count(const orc_sys *s);      /* canonical (symmetrised) count */
/* rows of (id_i, id_j, sx, sy, sz); image of j is pos_j + s*L */
int64_t orc_get_pairs(const orc_sys *s, int32_t *out5, int64_t cap);
int32_t orc_ghost_count(const orc_sys *s);
void orc_get_ghosts(const orc_sys *s, int32_t *src, int32_t *shift3, double *pos3);
/* Neighborlist::binlist_index of owned atoms then ghosts (cell-list mode). */
void orc_get_bins(const orc_sys *s, int32_t *owned3, int32_t *ghost3);
void orc_get_nbins(const orc_sys *s, int32_t *nb3);

/* Per-call pieces used by the tests. */
/* Shifted-force LJ potential of one pair (restated; see header). */
double orc_pair_potential(const orc_params *p, int32_t ti, int32_t tj, double r2);
/* Philox4x32-10 (Salmon et al., SC'11) on one counter block. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* Langevin noise of atom `id` at `step` (3 standard normals). */
void orc_langevin_eta(uint64_t seed, uint64_t step, uint32_t id, double eta[3]);

#ifdef __cplusplus
}
#endif
#endif
