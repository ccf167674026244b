/*
 * cavgpu.h -- C ABI of the GB300 (sm_103a) molecular-dynamics step of CAVIAR2.
 *
 * This is the drop-in boundary for the hot path of caviar-md/caviar-v2:
 * the Lennard-Jones pair force over a Verlet list, cell-list binning with a
 * half-skin-triggered list rebuild, and the velocity-Verlet and Langevin
 * integrate stages of Md_simulator.  Plain pointers and sizes only; every
 * host array uses the reference's own layouts (std::vector<Vector3d<double>>
 * is three contiguous doubles per atom, so `data()` passes as `const double*`
 * with stride 3; types and ids are size_t in Atom_struct and pass as
 * `const uint64_t*`).
 *
 * One context = one periodic system on one GPU, bound to one CUDA stream;
 * calls on one context are not thread-safe (the reference's Caviar2 object
 * is not re-entrant either).  There is no CPU fallback: without a GPU,
 * cavgpu_create returns CAVGPU_E_CUDA.
 *
 * Error convention: every call returns CAVGPU_OK (0) or a negative status;
 * cavgpu_strerror() names it.  The C++ host API above this layer turns the
 * statuses into the reference's behaviour (Log::error_all -> exit(1),
 * src/log.cpp:190-228; setters throw std::runtime_error, src/force/lj.cpp:76-77).
 */
#ifndef CAVGPU_H
#define CAVGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CAVGPU_MAX_TYPES 8

/* status codes */
#define CAVGPU_OK 0
#define CAVGPU_E_ARG -1            /* invalid argument or configuration */
#define CAVGPU_E_CUDA -2           /* CUDA runtime error or no device */
#define CAVGPU_E_NAN -3            /* NaN acceleration (src/md_simulator.cpp:646-652) */
#define CAVGPU_E_NLIST_OVERFLOW -4 /* neighbour capacity exceeded and could not grow */
#define CAVGPU_E_STATE -5          /* call out of order (e.g. step before upload) */
#define CAVGPU_E_NOMEM -6          /* device allocation failed */
#define CAVGPU_E_RANGE -7          /* size beyond a stated maximum */

/* precision of the pair force */
#define CAVGPU_FP64 0              /* all-FP64 kernels (the parity form) */
#define CAVGPU_MIXED 1             /* FP32 pair math on cell-relative coordinates, FP64 state */

/* integrators (Integrator_t, inc/caviar2/md_simulator.hpp:34-41) */
#define CAVGPU_VELOCITY_VERLET 0
#define CAVGPU_VELOCITY_VERLET_LANGEVIN 1
#define CAVGPU_LEAP_FROG 2             /* Md_simulator::integrate_leap_frog, src/md_simulator.cpp:871-980 */

typedef struct cavgpu_params {
  double lo[3], hi[3];            /* Domain::set_lower_global / set_upper_global */
  int32_t bc[3];                  /* Domain::set_boundary_condition; must be {1,1,1} */
  int32_t ntypes;                 /* 1..CAVGPU_MAX_TYPES */
  double nl_cutoff;               /* Neighborlist::set_cutoff */
  double nl_coef;                 /* Neighborlist::set_cutoff_extra_coef (>= 1) */
  double lj_cutoff;               /* force_field::Lj::set_cutoff */
  double eps[CAVGPU_MAX_TYPES * CAVGPU_MAX_TYPES];          /* Lj::set_epsilon, [ti*ntypes+tj] */
  double sigma[CAVGPU_MAX_TYPES * CAVGPU_MAX_TYPES];        /* Lj::set_sigma */
  double cutoff_list[CAVGPU_MAX_TYPES * CAVGPU_MAX_TYPES];  /* Lj::set_cutoff_list */
  int32_t cutoff_list_on;
  int32_t integrator;             /* CAVGPU_VELOCITY_VERLET, ..._LANGEVIN or CAVGPU_LEAP_FROG */
  double mass[CAVGPU_MAX_TYPES];  /* Atom_data::add_type_mass */
  double k_b;                     /* Atom_data::set_k_b */
  double dt;                      /* Md_simulator::set_dt */
  double lang_temperature;        /* Md_simulator::langevin_temperature */
  double lang_friction;           /* Md_simulator::langevin_friction */
  double lang_kb;                 /* Md_simulator::langevin_kb */
  double lang_kbt;                /* Md_simulator::langevin_kbt (<= 0: use kb*T) */
  uint64_t seed;                  /* Philox key of the Langevin noise */
  int32_t n_r_df;                 /* Atom_data::set_n_r_df, 0..3 */
  int32_t pressure_process;       /* Atom_data::set_pressure_process */
  int32_t precision;              /* CAVGPU_FP64 or CAVGPU_MIXED */
  int32_t noise_off;              /* Langevin with eta = 0 (exactness checks) */
  int32_t nbr_capacity;           /* neighbour slots per atom; 0 = sized at set-up */
  int32_t threads_per_atom;       /* force kernel lanes per atom (1,2,4,8,16); 0 = default */
  int32_t block_size;             /* force kernel block size (32..256, multiple of 32); 0 = default */
  int32_t steps_per_graph;        /* steps captured per CUDA graph; 0 = default (50); < 0 = no
                                     graphs, every kernel launched from the host (for profilers,
                                     which cannot see the kernels of graphs with conditional nodes) */
  int32_t force_kernel;           /* CAVGPU_FORCE_*: pair-kernel variant of the mixed form */
  double jump_tol;                /* Lj::set_jump_tol: r^2 of a pair inside the cutoff is floored at
                                     jump_tol (src/force/lj.cpp:459-468); 0 = off (the default) */
  int64_t initial_step;           /* Md_simulator::set_initial_step: index of the first step (the
                                     Philox step counter and the Nve schedule use it) */
  /* constraint::Nve velocity rescaling (src/constraint/nve.cpp:132-184): on every step whose
     index is a multiple of nve_step, velocities are scaled by lambda so that the kinetic
     energy becomes the target of nve_mode: after the closing kick and the temperature
     (velocity Verlet, leap-frog), or after the first half kick, before the atoms move
     (Langevin, src/md_simulator.cpp:782-793).  Single systems; 0 = off. */
  int64_t nve_step;
  int32_t nve_mode;               /* CAVGPU_NVE_ENERGY_PER_DOF, _ENERGY_TOT, _KBT, _KB_TEMPERATURE */
  int32_t nve_pad;
  double nve_value;               /* energy_per_dof, energy_tot, kbt or temperature */
  double nve_kb;                  /* kb of CAVGPU_NVE_KB_TEMPERATURE */
  /* Atom_data::msd_process (inc/caviar2/atom_data.hpp:690-700): count each atom's
   * periodic-boundary crossings per axis, as exchange_owned adds them to
   * Atom_struct::msd_domain_cross (src/atom_data/exchange_owned_single_md_domain.cpp:49-55) */
  int32_t msd_process;
  /* force_field::Lj::ignore_intra_molecule (src/force/lj.cpp:93-96, 446): pairs of atoms
   * with equal Atom_struct::molecule_index (cavgpu_set_molecules; -1 for every atom
   * until then, as Atom_data::add_atom sets it) take no force.  Applied when the
   * list is built, so cavgpu_export_pairs leaves those pairs out. */
  int32_t ignore_intra_molecule;
} cavgpu_params;

#define CAVGPU_NVE_ENERGY_PER_DOF 0
#define CAVGPU_NVE_ENERGY_TOT 1
#define CAVGPU_NVE_KBT 2
#define CAVGPU_NVE_KB_TEMPERATURE 3

/* pair-kernel variants of the mixed form (the FP64 form has one kernel); both give
 * the same results bit for bit */
#define CAVGPU_FORCE_AUTO 0       /* grid-strided; the autotuner may switch to segments */
#define CAVGPU_FORCE_STRIDED 1    /* grid-strided tasks, neighbour gathers from global memory */
#define CAVGPU_FORCE_SEGMENTS 2   /* row segments staged in shared memory */

typedef struct cavgpu_ctx cavgpu_ctx;

/* Fill *p with the reference's defaults (coef 1.12347, k_b 1, unit masses ...). */
void cavgpu_default_params(cavgpu_params *p);

/* Create a context on the current CUDA device.
 * Replaces: Caviar2 construction + Domain::generate (src/caviar2.cpp:20-28,
 * src/domain.cpp:295-307) for one periodic single-rank domain. */
int cavgpu_create(const cavgpu_params *p, cavgpu_ctx **out);
void cavgpu_destroy(cavgpu_ctx *ctx);

/* Upload n atoms (host order = insertion order; id defaults to the index).
 * pos3/vel3: Vector3d<double> arrays; type/id: Atom_struct size_t arrays.
 * Atoms must lie inside [lo, hi) (Atom_data::add_atom(tools::Atom&) rejects
 * others, src/atom_data/add_unique_atom_molecule.cpp:29-38).
 * Replaces: Atom_data::add_atom (src/atom_data.cpp:603-637). */
int cavgpu_upload(cavgpu_ctx *ctx, int64_t n, const double *pos3, const double *vel3, const uint64_t *type,
                  const uint64_t *id);

/* Per-atom molecule index in upload order (Atom_struct::molecule_index,
 * inc/caviar2/atom_data/utility/atom_struct.hpp:93), for
 * params.ignore_intra_molecule; after the upload, before cavgpu_setup. */
int cavgpu_set_molecules(cavgpu_ctx *ctx, const int32_t *molecule_index);

/* Initialise and set up: wrap, bin, build the list, first force, temperature.
 * Replaces: Md_simulator::initialize + setup (src/md_simulator.cpp:366-420, 565-611). */
int cavgpu_setup(cavgpu_ctx *ctx);

/* Advance nsteps steps of the configured integrator entirely on the device.
 * Replaces: Md_simulator::step / run loop (src/md_simulator.cpp:317-356, 445-546),
 * integrate_velocity_verlet (:617-729), integrate_velocity_verlet_langevin (:731-869),
 * re_calculate_acc (:422-437), Neighborlist::build (src/neighborlist.cpp:77-148). */
int cavgpu_step(cavgpu_ctx *ctx, int64_t nsteps);

/* Same as cavgpu_step, recording thermo every `every` steps into
 * out5[k*5 + {0..4}] = {KE, T, P, virialForce, PE} for k < nsteps/every.
 * Both calls return once the steps and the copies into out5 have completed.
 * The device status (NaN, list overflow) is read after every CUDA graph of steps:
 * a NaN acceleration returns CAVGPU_E_NAN with the steps before it done (the rest
 * of that graph does nothing; the context steps no further); a list that needs
 * more slots than it has is grown and the step completed from the same positions,
 * and the run goes on. */
int cavgpu_run(cavgpu_ctx *ctx, int64_t nsteps, int64_t every, double *out5);

/* Recompute the force at the current positions (list rebuilt if the half-skin
 * test asks for it) and return the virial and the potential energy.
 * Replaces: force_field::Lj::calculate_acceleration (src/force/lj.cpp:393-517). */
int cavgpu_forces(cavgpu_ctx *ctx, double *virial, double *pe);

/* out6 = {KE, T, P, virialForce, PE, rebuild count} of the last thermo point.
 * Replaces: Atom_data::kinetic_energy / temperature / pressure
 * (src/atom_data/kinetic_energy.cpp:26-303). */
int cavgpu_thermo(cavgpu_ctx *ctx, double *out6);

/* Download in host (insertion) order; positions wrapped as Domain::fix_position
 * would (src/domain.cpp:443-493).  Any pointer may be NULL. */
int cavgpu_download(cavgpu_ctx *ctx, double *pos3, double *vel3, double *acc3);

/* Boundary crossings per atom and axis in host order (int32 x3), counted since
 * the upload: +1 through the upper face, -1 through the lower, including the wrap
 * Domain::fix_position would apply to the current position (src/domain.cpp:443-493).
 * Needs params.msd_process.
 * Replaces: reading Atom_struct::msd_domain_cross (inc/caviar2/atom_data/utility/atom_struct.hpp:86). */
int cavgpu_download_images(cavgpu_ctx *ctx, int32_t *img3);

/* Canonical pair set of the current list: rows (id_i, id_j, sx, sy, sz), the
 * image of j being pos_j + s*L; both orders of every pair.  Returns the row
 * count (negative on error); writes at most cap rows.
 * Replaces: Neighborlist::neighlist (inc/caviar2/neighborlist.hpp:102). */
int64_t cavgpu_export_pairs(cavgpu_ctx *ctx, int32_t *out5, int64_t cap);

/* Reference cell assignment of every atom (host order) at the current
 * positions: Neighborlist::binlist_index (src/neighborlist.cpp:392-414) with
 * no_bins = ceil(L / cutoff_extra) (src/neighborlist.cpp:336-342). */
int cavgpu_export_bins(cavgpu_ctx *ctx, int32_t *owned3, int32_t *nbins3);

/* Periodic images in the reference's ghost order (owned atom by atom; face,
 * edge, corner images x, y, z, xy, xz, yz, xyz) for a ghost cutoff, with their
 * reference bins.  Returns the ghost count; writes at most cap entries.
 * Replaces: Atom_data::exchange_ghost_single_md_domain
 * (src/atom_data/exchange_ghost_single_md_domain.cpp:24-215). */
int64_t cavgpu_export_ghosts(cavgpu_ctx *ctx, double ghost_cutoff, int32_t *src, int32_t *shift3, double *pos3,
                             int32_t *bins3, int64_t cap);

/* Statistics: out8 = {steps done, rebuilds, max neighbours, capacity,
 * threads per atom, block size, graph launches, kernel launches}. */
int cavgpu_stats(cavgpu_ctx *ctx, int64_t *out8);

/* The CUDA stream the context launches on (a cudaStream_t). */
void *cavgpu_stream(cavgpu_ctx *ctx);

/* Kernel timing: when on, CUDA events bracket every force-kernel launch (on
 * the context's stream, also inside captured graphs) and the totals
 * accumulate until read.  out: {force launches, force ms total}. */
int cavgpu_set_profiling(cavgpu_ctx *ctx, int32_t on);
int cavgpu_read_profile(cavgpu_ctx *ctx, double *out2);

const char *cavgpu_strerror(int status);

/* Text of the last CUDA runtime error this library saw on the calling thread
 * ("none" if none); complements CAVGPU_E_CUDA (the reference logs the reason
 * before exiting, src/log.cpp:190-228). */
const char *cavgpu_last_cuda_error(void);

/* Kinetic energy and temperature of n atoms held in caller-owned DEVICE memory,
 * without any device allocation (no counterpart in the reference; the result is
 * that of Atom_data::kinetic_energy / finalize_temperature for n_r_df 0..3).
 * For callers that cannot call cudaMalloc: work enqueued inside a CUDA-graph
 * stream capture, memory owned by another allocator, loops that must not
 * synchronise.  vel3: 3 doubles per atom; type: uint64 per atom (types >= ntypes
 * count as massless); mass: HOST array of ntypes masses; out2: DEVICE array that
 * receives {KE, T} when `stream` (a cudaStream_t, NULL = legacy default) reaches it.
 * Scratch: a fixed 320 KiB __device__ array (per-block partial sums) that every
 * device loading this library keeps until exit; n > 16,777,216 returns
 * CAVGPU_E_RANGE.  The first call on a device looks up that array's device
 * address once; make that first call before any stream capture.  The address is
 * kept for the life of the process: after cudaDeviceReset it is stale, so do not
 * call this on a device that was reset.  Calls share the array: two calls that
 * overlap on the GPU race. */
int cavgpu_kinetic_energy_noalloc(int64_t n, const double *vel3, const uint64_t *type, const double *mass,
                                  int32_t ntypes, int32_t n_r_df, double k_b, double *out2, void *stream);

/* Autotuner (no counterpart in the reference, whose loop has no launch shape):
 * times short trial runs of every launch shape -- pair kernel (mixed form with
 * CAVGPU_FORCE_AUTO: segments and grid-strided) x force-kernel lanes per atom
 * {1,2,4,8} x block size {64,128,256}, then steps per captured graph {25,50,100}
 * -- each started from a snapshot of the current state, and keeps the fastest.
 * The state afterwards is the snapshot's (positions, velocities, accelerations,
 * step counter, statistics), with the list rebuilt for the chosen shape; the
 * changed summation order perturbs later FP64 results at rounding level, as any
 * launch-shape change does.  trial_steps: steps timed per candidate (0 = 40).
 * Results are cached per process by (device, precision, integrator, replica
 * count, atom count, type count, force_kernel); CAVGPU_TUNE_FORCE re-measures.
 * out6 (may be NULL) = {threads per atom, block size, steps per graph, trials,
 * pair kernel (CAVGPU_FORCE_STRIDED or _SEGMENTS), 0}. */
#define CAVGPU_TUNE_FORCE 1
int cavgpu_autotune(cavgpu_ctx *ctx, int32_t trial_steps, int32_t flags, int64_t *out6);

/* ---- batches of independent replicas (no counterpart in the reference: one
 * CAVIAR2 process runs one Md_simulator; a batch is R of them in one context,
 * each with its own periodic box, atom count, cell grid and half-skin rebuild,
 * sharing params, pair table and integrator).  A batch advances with
 * cavgpu_step / cavgpu_run(every = 0) and each replica's trajectory equals that
 * of its own single-system context in FP64 form.  The single-system exports
 * (pairs, bins, ghosts) and cavgpu_thermo refuse batches (CAVGPU_E_ARG). */

/* Create a batch of nrep >= 1 replicas; replica r's box is [lo3[3r..3r+2],
 * hi3[3r..3r+2]) (p->lo / p->hi are ignored); each edge >= 2 (nl_cutoff * nl_coef). */
int cavgpu_create_batch(const cavgpu_params *p, int32_t nrep, const double *lo3, const double *hi3,
                        cavgpu_ctx **out);

/* Upload counts[r] >= 1 atoms per replica, concatenated in replica order
 * (pos3/vel3: 3 doubles per atom; vel3 may be NULL; type: uint64 per atom).
 * download returns the atoms in the same concatenated order. */
int cavgpu_upload_batch(cavgpu_ctx *ctx, const int64_t *counts, const double *pos3, const double *vel3,
                        const uint64_t *type);

/* Per-replica thermo of the last thermo point: out6[6r + {0..5}] = {KE, T, P,
 * virialForce, PE, total mass} (Atom_data::kinetic_energy / temperature /
 * pressure of replica r alone). */
int cavgpu_thermo_batch(cavgpu_ctx *ctx, double *out6);

/* Diagnostic (no counterpart in the reference): measured FMA throughput of the
 * current device, out2 = {FP64 TFLOP/s, FP32 TFLOP/s}, for roofline denominators. */
int cavgpu_measure_peaks(double *out2);

#ifdef __cplusplus
}
#endif
#endif
