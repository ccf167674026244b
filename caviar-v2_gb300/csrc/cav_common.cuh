// cav_common.cuh -- device state, constants and small device helpers shared by
// the sm_103a kernels of the CAVIAR2 MD step.
//
// One context holds R >= 1 independent periodic systems ("replicas"); a single
// system is R = 1.  Replica r owns a contiguous, 32-aligned range of atom slots
// (so that no warp of any kernel straddles two replicas) and a contiguous range
// of search cells; the slots after its atoms, up to the next aligned start, are
// padding that no kernel updates and no list refers to.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cavgpu.h"

namespace cav {

// 32-byte aligned 4-vector of doubles: one 256-bit access per atom
typedef double4_32a dbl4;
__host__ __device__ inline dbl4 make_dbl4(double x, double y, double z, double w) {
  dbl4 r;
  r.x = x; r.y = y; r.z = z; r.w = w;
  return r;
}
// The atom type rides in the w component of its position as the integer's bit
// pattern (not as a double value): reading it back is integer work, off the FP64
// pipe the FP64 pair loop is bound by.
__host__ __device__ inline double type_bits(int t) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)t);
#else
  double r;
  const long long v = t;
  static_assert(sizeof(r) == sizeof(v), "64-bit double");
  __builtin_memcpy(&r, &v, sizeof(r));
  return r;
#endif
}
__device__ inline int type_of(const double w) { return (int)__double_as_longlong(w); }

// read-only (non-coherent) 256-bit load of a neighbour's position
__device__ inline dbl4 ldg_dbl4(const dbl4 *p) {
  dbl4 r;
  asm("ld.global.nc.v4.f64 {%0,%1,%2,%3}, [%4];" : "=d"(r.x), "=d"(r.y), "=d"(r.z), "=d"(r.w) : "l"(p));
  return r;
}

constexpr int MAXT = CAVGPU_MAX_TYPES;
constexpr int THERMO_REC = 5;  // {KE, T, P, virialForce, PE} per recorded step
// neighbour entry: bits 0..26 = atom slot j, bits 27..31 = image code (0..26)
constexpr int CODE_SHIFT = 27;
constexpr uint32_t IDX_MASK = (1u << CODE_SHIFT) - 1u;
constexpr int64_t MAX_ATOMS = (int64_t)IDX_MASK;  // 134,217,727 slots
constexpr int CODE_ZERO = 13;                      // (0,0,0)
constexpr int SLOT_ALIGN = 32;                     // replica slot ranges start on warp boundaries

// device flag words
enum Flag : int {
  F_REBUILD = 0,    // some replica must rebuild its list before the next force (half-skin test fired)
  F_MAXNB = 1,      // largest neighbour count seen by the last build
  F_OVERFLOW = 2,   // a build wanted more than `cap` slots
  F_NAN = 3,        // NaN acceleration seen
  F_NAN_ATOM = 4,   // host index of one NaN atom
  F_REBUILDS = 5,   // replica list builds (a single system: its rebuild count)
  F_PASSES = 6,     // rebuild passes that built at least one replica
  // Halt: raised after a list overflow or a NaN, only by single points of a step
  // (the condition kernel, the pair kernel's last block, the end of a rebuild), so
  // that it is constant while any kernel runs; every step kernel that starts with
  // it raised returns at once, and the rest of the chunk does nothing.
  F_HALT = 7,
  F_STEPS_OK = 8,   // steps of the current chunk whose pair kernel ran (the step counter adds them)
  F_HALT_STEP = 9,  // steps of the halted chunk that completed before the halt
  F_UPLOAD_BAD = 10,  // an uploaded atom outside the box, of an unknown type or with a bad id
  F_NWORDS = 12
};

// what the pair kernel does after the closing update of its step: nothing, or the
// first half of the next step (its drift), so that one launch serves one step
enum Fuse : int { FUSE_NONE = 0, FUSE_VV = 1, FUSE_LF = 2, FUSE_LANG = 3 };

// Per type-pair constants of the shifted-force LJ (force_field::Lj,
// src/force/lj.cpp:470-484).  For r^2 <= rc2:
//   coef(r) = g(r) - g(rc),  g(r) = eps4 * s6 * (6 - 12 s6) / r^2,  s6 = (sig2/r^2)^3
//   V(r)    = eps4 (s6^2 - s6) - uc - gc/2 (r^2 - rc2),  gc = g(rc), uc = U(rc)
// rc2 < 0 marks an eps == 0 pair (skipped, src/force/lj.cpp:471-472).
struct PairTab {
  double rc2[MAXT * MAXT], sig2[MAXT * MAXT], eps4[MAXT * MAXT], gc[MAXT * MAXT], uc[MAXT * MAXT];
  double minv[MAXT], mass[MAXT];
  int nt;
};

// One replica's periodic box and search grid.
struct RepBox {
  double lo[3], hi[3], L[3];
  double w[3], inv_w[3];  // search cell width >= list cutoff
  float wf[3];            // cell width rounded to FP32 ...
  float wlo[3];           // ... and the rest, w - wf (a cell offset is d*wf + d*wlo in the mixed form)
  int nc[3];
  int cell_off, ncell;    // cells [cell_off, cell_off + ncell); cell cell_off + ncell holds the padding
  int slot_off, natoms, pad;
  int id_off;             // host index of the replica's first atom; atom ids are local (0..natoms-1)
};

// Batch-wide geometry (by value in every launch).
struct Box {
  const RepBox *rep;    // [nrep] (device)
  const int *rep_of;    // slot -> replica, -1 for padding (device; null when nrep == 1)
  const int *cell_rep;  // cell -> replica, -1 for a padding cell (device; null when nrep == 1)
  int *rep_flag;        // per replica: rebuild requested (device)
  int nrep, nslot, ncell_all;  // ncell_all counts the padding cells
  double ce2;           // cutoff_extra^2, the list predicate r^2 < ce2 (src/neighborlist.cpp:258, :508)
  float ce2_lo, ce2_hi; // FP32 pre-screen band around ce2
  double thr2;          // 0.25 (cutoff_extra - cutoff)^2 (src/neighborlist.cpp:318)
  float thr2f;          // thr2 * (1 - 1e-6) in FP32: the mixed form's test may only fire early
  RepBox r0;            // replica 0 by value: the single-system path reads no replica table
};

__device__ inline const RepBox &repbox(const Box &b, int r) { return b.nrep == 1 ? b.r0 : b.rep[r]; }
__device__ inline int rep_of_slot(const Box &b, int i) { return b.nrep == 1 ? 0 : b.rep_of[i]; }
__device__ inline int rep_of_cell(const Box &b, int c) { return b.nrep == 1 ? (c < b.r0.ncell ? 0 : -1) : b.cell_rep[c]; }

struct StepConsts {
  double dt, hdt, hdt2;       // dt, 0.5*dt, 0.5*dt*dt
  double la, lb, lc;          // Langevin a, b, c (src/md_simulator.cpp:398-405)
  uint64_t seed;
  int noise_off;
  int n;                      // slots
  double jump_tol;            // Lj jump_fix: floor of r^2 inside the cutoff (0 = off)
  float jump_tolf;
};

// Device arrays, in cell-sorted slot order.
struct Dev {
  // acc holds a(t) from the pair kernel until the next pair kernel replaces it, so
  // the velocity-Verlet kick reads it as a_old (leap-frog's drift zeroes it)
  dbl4 *pos, *vel, *acc, *pos_ref;
  float4 *rel;                // position relative to the build cell's origin; w = type bits
  float4 *rel_ref;            // rel at the last build (mixed form: rel = rel_ref + (x - pos_ref))
  // the coordinates a pair kernel gathers from its neighbours, for the next step: a pair
  // kernel that also drifts its atoms writes them here (FP64 form: positions; mixed
  // form: rel), while other atoms still read the current ones, and the two swap
  dbl4 *pos_alt;
  float4 *rel_alt;
  unsigned int *force_ticket; // pair kernel: blocks done (the last one ends the step and resets it)
  int *type;
  uint32_t *id;               // host (insertion) index
  int *cell_of;               // build cell of each slot
  int4 *img;                  // periodic-boundary crossings per axis (msd_domain_cross); null when not tracked
  int *mol;                   // molecule index (ignore_intra_molecule); null when off
  // rebuild scratch
  dbl4 *t_pos, *t_vel, *t_acc;
  int *t_type;
  uint32_t *t_id;
  int4 *t_img;
  int *t_mol;
  int *atom_cell, *cell_count, *cell_start, *cell_cursor, *perm, *perm_tmp;
  uint64_t *skey;             // order inside a cell: Morton index of the 4x4x4 sub-cell, then id
  // neighbour list
  uint32_t *nbr;
  int *nnbr;
  int cap;                    // slots per atom (multiple of 64)
  int tpa;                    // force-kernel lanes per atom (fixes the list layout)
  // status, reductions
  int *flags;
  double *partials_ke;        // per-block {sum m v^2, sum m v} (4 per block)
  double *partials_ke_end;    // Langevin: the same sums over the velocities at the end of the step
  double *partials_ev;        // per-block {sum -coef r^2, sum V} over both pair orders (2 per block)
  int partials_blocks;        // blocks the partial arrays hold (every launch grid is checked against it)
  double2 *ev_atom;           // per-slot {-coef r^2, V} sums (batches: per-replica folds)
  double *thermo;             // {KE, T, P, virialForce, PE, total mass, -, -}
  double *thermo_rep;         // batches: per replica {KE, T, P, virialForce, PE, total mass, -, -}
  double *thermo_ring;        // recorded thermo points (THERMO_REC per record)
  long long *step_base;       // index of the chunk's first step (Langevin noise, Nve schedule)
  double *nve_partials;       // Nve: per-block {sum m v^2, sum m v} (4 per block, NVE_BLOCKS blocks)
  int *scan_part;             // single system: counts per scan slice (SCAN_SLICES)
  double *fold;               // thermo fold: per-block sums of the first level (THERMO_FOLD_BLOCKS x 10)
  unsigned int *fold_ticket;  // thermo fold: blocks done (the last one folds and resets it to 0)
  double *nve_lambda;         // Nve: the scale factor of the current step
  PairTab *tab;
  // host-order staging for downloads
  double *h3;
  int32_t *hi3;
  // row segments of the mixed force kernel: {replica, cy | cz << 16, first cell x, cells}
  const int4 *seg;
  int nseg;
  int seg_umax;               // most cells a segment stages per row (segment length + 2)
  int stage_cap;              // staged atoms the shared memory holds (float4 each)
};

// Dynamic shared memory of the segment force kernel: the staged coordinates, then
// two int tables of 9 rows x seg_umax cells (slot offset, count).
inline size_t seg_smem_bytes(int stage_cap, int umax) {
  return (size_t)stage_cap * 16 + (size_t)2 * 9 * umax * sizeof(int);
}

// ---- neighbour-list layout -------------------------------------------------
// A warp of the force kernel serves A = 32/tpa atoms (a block of A consecutive
// slots).  Within a block, entries come in chunks of four: chunk g of atom i
// holds entries 4g..4g+3 at block_base + g*4A + (i % A)*4.  Force-kernel lane
// (t, a) reads chunks g = t + tpa*q with one 128-bit load, so a warp reads 512
// consecutive bytes per step of q.  A and tpa are powers of two: shifts only.
// `cap` is a multiple of 4*tpa (64 covers every tpa up to 16).
__host__ __device__ inline int log2_pow2(int v) {
#ifdef __CUDA_ARCH__
  return __ffs(v) - 1;
#else
  return __builtin_ctz((unsigned)v);
#endif
}
__host__ __device__ inline size_t nbr_block_base(int i, int cap, int tpa) {
  const int as = 5 - log2_pow2(tpa);  // log2(A)
  return ((size_t)(i >> as) * (size_t)cap << as) + ((size_t)(i & ((1 << as) - 1)) << 2);
}
__host__ __device__ inline size_t nbr_index(int i, int k, int cap, int tpa) {
  const int as = 5 - log2_pow2(tpa);
  return nbr_block_base(i, cap, tpa) + ((size_t)(k >> 2) << (as + 2)) + (k & 3);
}

__host__ __device__ inline int image_code(int sx, int sy, int sz) { return (sx + 1) + 3 * (sy + 1) + 9 * (sz + 1); }

// ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) -----------------------
__device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += W0; k1 += W1; }
    const uint32_t hi0 = __umulhi(M0, c[0]), lo0 = M0 * c[0];
    const uint32_t hi1 = __umulhi(M1, c[2]), lo1 = M1 * c[2];
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
  }
}

constexpr uint32_t LANG_TAG = 0x4C414E47u;

// Langevin noise of atom `id` at `step`: Box-Muller on one Philox block (FP64).
__device__ inline void langevin_eta(uint64_t seed, long long step, uint32_t id, double &e0, double &e1, double &e2) {
  uint32_t c[4] = {(uint32_t)step, (uint32_t)((unsigned long long)step >> 32), id, LANG_TAG};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  const double s = 2.3283064365386963e-10;  // 2^-32
  const double u0 = ((double)c[0] + 0.5) * s, u1 = ((double)c[1] + 0.5) * s;
  const double u2 = ((double)c[2] + 0.5) * s, u3 = ((double)c[3] + 0.5) * s;
  const double r0 = sqrt(-2.0 * log(u0)), r1 = sqrt(-2.0 * log(u2));
  double sn, cs;
  sincospi(2.0 * u1, &sn, &cs);
  e0 = r0 * cs;
  e1 = r0 * sn;
  e2 = r1 * cospi(2.0 * u3);
}

// FP32 variant for the mixed-precision form (noise precision is immaterial).
__device__ inline void langevin_eta_f(uint64_t seed, long long step, uint32_t id, double &e0, double &e1,
                                      double &e2) {
  uint32_t c[4] = {(uint32_t)step, (uint32_t)((unsigned long long)step >> 32), id, LANG_TAG};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  const float s = 2.3283064365386963e-10f;
  const float u0 = ((float)c[0] + 0.5f) * s, u1 = ((float)c[1] + 0.5f) * s;
  const float u2 = ((float)c[2] + 0.5f) * s, u3 = ((float)c[3] + 0.5f) * s;
  const float r0 = sqrtf(-2.0f * logf(fmaxf(u0, 1e-30f))), r1 = sqrtf(-2.0f * logf(fmaxf(u2, 1e-30f)));
  float sn, cs;
  sincospif(2.0f * u1, &sn, &cs);
  e0 = (double)(r0 * cs);
  e1 = (double)(r0 * sn);
  e2 = (double)(r1 * cospif(2.0f * u3));
}

// ---- integrator arithmetic shared by the drift kernels and the pair kernel ----
// FP64 form: the reference's expression orders (src/md_simulator.cpp:654, 898-899,
// 765, 822-827), no contraction, so that equal forces give equal trajectories.
// Mixed form: FMAs (the FP64 pipe of these updates is their scarcest resource).

// velocity Verlet: pos += vel*dt + ((acc*0.5)*dt)*dt
template <bool MIXED>
__device__ __forceinline__ void drift_vv(dbl4 &x, const dbl4 &v, const dbl4 &a, const StepConsts &sc) {
  if (MIXED) {
    x.x = fma(a.x, sc.hdt2, fma(v.x, sc.dt, x.x));
    x.y = fma(a.y, sc.hdt2, fma(v.y, sc.dt, x.y));
    x.z = fma(a.z, sc.hdt2, fma(v.z, sc.dt, x.z));
  } else {
    x.x = __dadd_rn(x.x, __dadd_rn(__dmul_rn(v.x, sc.dt), __dmul_rn(__dmul_rn(__dmul_rn(a.x, 0.5), sc.dt), sc.dt)));
    x.y = __dadd_rn(x.y, __dadd_rn(__dmul_rn(v.y, sc.dt), __dmul_rn(__dmul_rn(__dmul_rn(a.y, 0.5), sc.dt), sc.dt)));
    x.z = __dadd_rn(x.z, __dadd_rn(__dmul_rn(v.z, sc.dt), __dmul_rn(__dmul_rn(__dmul_rn(a.z, 0.5), sc.dt), sc.dt)));
  }
}

// leap-frog first half: v += (0.5 dt) a ; r += dt v
template <bool MIXED>
__device__ __forceinline__ void drift_lf(dbl4 &x, dbl4 &v, const dbl4 &a, const StepConsts &sc) {
  if (MIXED) {
    v.x = fma(a.x, sc.hdt, v.x); v.y = fma(a.y, sc.hdt, v.y); v.z = fma(a.z, sc.hdt, v.z);
    x.x = fma(v.x, sc.dt, x.x); x.y = fma(v.y, sc.dt, x.y); x.z = fma(v.z, sc.dt, x.z);
  } else {
    v.x = __dadd_rn(v.x, __dmul_rn(sc.hdt, a.x));
    v.y = __dadd_rn(v.y, __dmul_rn(sc.hdt, a.y));
    v.z = __dadd_rn(v.z, __dmul_rn(sc.hdt, a.z));
    x.x = __dadd_rn(x.x, __dmul_rn(sc.dt, v.x));
    x.y = __dadd_rn(x.y, __dmul_rn(sc.dt, v.y));
    x.z = __dadd_rn(x.z, __dmul_rn(sc.dt, v.z));
  }
}

// Langevin first half, velocity part: v += (a*0.5)*dt + eta*b
template <bool MIXED>
__device__ __forceinline__ void lang_half(dbl4 &v, const dbl4 &a, double e0, double e1, double e2,
                                          const StepConsts &sc) {
  if (MIXED) {
    v.x = fma(a.x, sc.hdt, fma(e0, sc.lb, v.x));
    v.y = fma(a.y, sc.hdt, fma(e1, sc.lb, v.y));
    v.z = fma(a.z, sc.hdt, fma(e2, sc.lb, v.z));
  } else {
    v.x = __dadd_rn(v.x, __dadd_rn(__dmul_rn(__dmul_rn(a.x, 0.5), sc.dt), __dmul_rn(e0, sc.lb)));
    v.y = __dadd_rn(v.y, __dadd_rn(__dmul_rn(__dmul_rn(a.y, 0.5), sc.dt), __dmul_rn(e1, sc.lb)));
    v.z = __dadd_rn(v.z, __dadd_rn(__dmul_rn(__dmul_rn(a.z, 0.5), sc.dt), __dmul_rn(e2, sc.lb)));
  }
}

// Langevin position update r += v*c
template <bool MIXED>
__device__ __forceinline__ void lang_move(dbl4 &x, const dbl4 &v, const StepConsts &sc) {
  if (MIXED) {
    x.x = fma(v.x, sc.lc, x.x); x.y = fma(v.y, sc.lc, x.y); x.z = fma(v.z, sc.lc, x.z);
  } else {
    x.x = __dadd_rn(x.x, __dmul_rn(v.x, sc.lc));
    x.y = __dadd_rn(x.y, __dmul_rn(v.y, sc.lc));
    x.z = __dadd_rn(x.z, __dmul_rn(v.z, sc.lc));
  }
}

__device__ inline void request_rebuild(const Dev &d, const Box &b, int rep) {
  b.rep_flag[rep] = 1;
  d.flags[F_REBUILD] = 1;
}

// Half-skin test of the reference (src/neighborlist.cpp:134-143), FP64 form.
__device__ inline void half_skin_test(const Dev &d, const Box &b, int rep, int i, const dbl4 &x) {
  const dbl4 r = d.pos_ref[i];
  const double dx = x.x - r.x, dy = x.y - r.y, dz = x.z - r.z;
  if (dx * dx + dy * dy + dz * dz > b.thr2) request_rebuild(d, b, rep);
}

// Mixed form: the displacement since the build is taken once in FP64 (3
// subtractions) and serves both the half-skin test (in FP32 against a threshold
// shrunk by 1e-6, so it can only fire early) and the FP32 cell-relative
// coordinates, rel = rel_at_build + (float)(x - x_at_build), written to rel_out.
__device__ inline void mixed_track(const Dev &d, const Box &b, int rep, int i, const dbl4 &x, float4 *rel_out) {
  const dbl4 r = d.pos_ref[i];
  const float fx = (float)(x.x - r.x), fy = (float)(x.y - r.y), fz = (float)(x.z - r.z);
  if (fx * fx + fy * fy + fz * fz > b.thr2f) request_rebuild(d, b, rep);
  const float4 q = d.rel_ref[i];
  rel_out[i] = make_float4(q.x + fx, q.y + fy, q.z + fz, q.w);
}

__device__ inline void nan_check(const Dev &d, int i, const dbl4 &a) {
  if (isnan(a.x) || isnan(a.y) || isnan(a.z)) {
    d.flags[F_NAN] = 1;
    d.flags[F_NAN_ATOM] = (int)d.id[i];
  }
}

// the halt word as every thread of a kernel sees it (constant while kernels run)
__device__ inline bool halted(const Dev &d) { return *(volatile const int *)&d.flags[F_HALT] != 0; }

// ---- host-side launch helpers ----------------------------------------------
struct LaunchCfg {
  int precision;   // CAVGPU_FP64 / CAVGPU_MIXED
  int integrator;  // CAVGPU_VELOCITY_VERLET / ..._LANGEVIN
  int tpa, block;
  int n;           // slots
  int nseg;        // row segments (mixed form; 0 = none)
  int use_seg;     // mixed form: run the segment kernel (shared-memory stage)
  int ntypes;      // 1: the mixed kernels keep the pair constants in registers
};

struct ThermoCfg {
  int n_r_df;
  double k_b, volume;
  int n;           // atoms (single system)
  int langevin;    // pressure without the force virial (the reference computes it before the force)
};

// KE, T, P, virial, PE from the folded sums (Atom_data::kinetic_energy_mpi_domain /
// finalize_temperature / finalize_pressure, src/atom_data/kinetic_energy.cpp:26-134,
// 189-198, 238-303)
__device__ inline void thermo_finish(double ke2, const double P3[3], double msum, double vir2, double pe2, int natoms,
                                     int n_r_df, double k_b, double volume, int langevin, double *out) {
  if (n_r_df >= 1 && n_r_df <= 3 && msum > 0) ke2 -= (P3[0] * P3[0] + P3[1] * P3[1] + P3[2] * P3[2]) / msum;
  const double ke = 0.5 * ke2;
  const int dof = 3 * natoms - n_r_df;
  const double T = 2.0 * ke / (k_b * dof);
  const double vir = 0.5 * vir2;  // each pair was visited from both sides
  out[0] = ke;
  out[1] = T;
  out[2] = ((double)natoms * k_b * T) / volume + (langevin ? 0.0 : vir) / (3.0 * volume);
  out[3] = vir;
  out[4] = 0.5 * pe2;
}

// Kernel launchers (cav_kernels.cu, cav_force.cu).  `forced` rebuilds every
// replica regardless of the flags; otherwise the rebuild kernels skip replicas
// whose half-skin test did not fire.
int drift_grid_blocks(const LaunchCfg &lc);
int force_grid_blocks(const LaunchCfg &lc);
// sets the dynamic shared-memory limit of every segment-kernel variant (call outside capture)
int prepare_force_seg(size_t smem_bytes);
// thermo < 0 (Langevin): the velocity half only; launch_lang_pos then moves the atoms
int launch_drift(const Dev &d, const Box &b, const StepConsts &sc, const LaunchCfg &lc, int k_in_chunk,
                 int thermo, cudaStream_t st);
int launch_lang_pos(const Dev &d, const Box &b, const StepConsts &sc, const LaunchCfg &lc, int thermo,
                    cudaStream_t st);
int launch_rebuild(const Dev &d, const Box &b, const LaunchCfg &lc, int forced, cudaStream_t st);
int launch_set_rebuild_cond(const Dev &d, cudaGraphConditionalHandle h, cudaStream_t st);
// steps launched from the host: a NaN the drift saw halts the chunk
int launch_halt_check(const Dev &d, cudaStream_t st);
// a single system scans its cell counts in SCAN_SLICES slices (one more kernel)
constexpr int SCAN_SLICES = 64;
inline int scan_slices(const Box &b) { return b.nrep == 1 ? SCAN_SLICES : 1; }
// kernels launch_rebuild enqueues
inline int rebuild_kernels(const Box &b) { return 8 + (scan_slices(b) > 1 ? 1 : 0); }
// kick: 0 = force only, 1 = VV closing kick, 2 = Langevin closing update.
// thermo: virial/PE partials (and KE partials unless kick == 2).
// fuse (Fuse): the next step's drift in the same launch, written to d.pos_alt (FP64)
// or d.rel_alt (mixed); the caller swaps them with d.pos / d.rel afterwards.
// cond: when set_cond, the last block sets the conditional node of the next step's
// rebuild to the half-skin flag (unless halted).  The last block also counts the
// step (F_STEPS_OK) and raises the halt on a NaN.
// The thermo fold of a recorded step done by the pair kernel's last block (single
// systems): the fixed-order sums of the KE partials (nb_ke blocks; Langevin: the
// drift kernel's) and of the launch's own virial/PE partials (and, Langevin, of its
// end-of-step KE partials, nb_ke_end), then the record -- what launch_thermo_final
// does after the launch, without its launch.
struct FoldArgs {
  ThermoCfg tc;
  int nb_ke, nb_ke_end, ring_slot;
};
int launch_force(const Dev &d, const Box &b, const StepConsts &sc, const LaunchCfg &lc, int kick, int thermo,
                 int k_in_chunk, int fuse, int set_cond, cudaGraphConditionalHandle cond, cudaStream_t st,
                 const FoldArgs *fold = nullptr);
// nb_ke_end > 0 (Langevin): KE from partials_ke_end, the temperature from partials_ke.
// Two levels in a fixed order: THERMO_FOLD_BLOCKS blocks fold strided subsets of the
// partials, the last block to finish folds their sums (deterministic).
constexpr int THERMO_FOLD_BLOCKS = 32;
int launch_thermo_final(const Dev &d, const ThermoCfg &tc, int nb_ke, int nb_ev, int nb_ke_end, int ring_slot,
                        cudaStream_t st);
// batches: per-replica KE (ke = 1, from the current velocities) and/or virial+PE folds
int launch_thermo_replicas(const Dev &d, const Box &b, const ThermoCfg &tc, int ke, int ev, cudaStream_t st);
int launch_advance_step(const Dev &d, cudaStream_t st);
// constraint::Nve: kinetic energy, lambda (and the thermo point of the step,
// ring_slot >= 0 or the current one when thermo != 0), velocity scaling; every
// kernel returns at once unless (step_base + k) % cfg.step == 0
struct NveCfg {
  long long step;
  int mode;
  double value, kb;
};
constexpr int NVE_BLOCKS = 1024;
int launch_nve(const Dev &d, const Box &b, const ThermoCfg &tc, const NveCfg &cfg, int k, int thermo, int ring_slot,
               cudaStream_t st);
int launch_to_host_order(const Dev &d, const Box &b, int what, cudaStream_t st);
// boundary crossings per atom in host order into d.hi3, counting the wrap of the
// current position that the next list build applies
int launch_images_to_host(const Dev &d, const Box &b, cudaStream_t st);
int launch_export_pairs(const Dev &d, const Box &b, int mode, int32_t *rows, unsigned long long *counter,
                        int64_t cap, cudaStream_t st);
int launch_ref_bins(const Dev &d, int n, double cutoff_inv, const int nb[3], const double lo_local[3],
                    cudaStream_t st);
// Single system: the host arrays as the caller passed them (pos3, vel3 doubles; type,
// id uint64), copied raw into the rebuild scratch, become the slot arrays; every atom
// is checked as Atom_data::add_atom(tools::Atom &) checks it (inside [lo, hi)), its
// type and id too; F_UPLOAD_BAD is raised for a bad atom.  type_count[t] counts the
// atoms of each type (exact integers: the total mass follows in a fixed order).
int launch_upload_single(const Dev &d, const Box &b, int n, int ntypes, bool has_vel, bool has_id,
                         const double *raw_pos, const double *raw_vel, const uint64_t *raw_type,
                         const uint64_t *raw_id, int *seen, int *type_count, cudaStream_t st);
int launch_ghosts(const Dev &d, const Box &b, int n, double gc, int *counts, int *starts, int32_t *src,
                  int32_t *shift3, double *pos3, int32_t *bins3, int64_t cap, double cutoff_inv, const int nb[3],
                  const double lo_local[3], cudaStream_t st);

}  // namespace cav
