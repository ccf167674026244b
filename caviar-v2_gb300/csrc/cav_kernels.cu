// cav_kernels.cu -- sm_103a kernels of the CAVIAR2 MD step (integrator stages,
// cell binning, Verlet-list build, thermo reductions, parity exports).  The
// pair-force kernels live in cav_force.cu.  Every kernel serves R >= 1 replicas
// (see cav_common.cuh); a single system is R = 1.
#include <algorithm>

#include "cav_common.cuh"

namespace cav {

#define FULL_MASK 0xffffffffu

static inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

static int num_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 148;
  }
  return sms;
}

// ---------------------------------------------------------------------------
// block reduction of NV doubles in a fixed order (deterministic)
// ---------------------------------------------------------------------------
template <int NV>
__device__ inline void block_sum_store(double (&v)[NV], double *out /* NV doubles */) {
  __shared__ double sh[32][NV];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(FULL_MASK, v[k], o);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[wid][k] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < NV; ++k) {
      double s = 0.0;
      for (int w = 0; w < nw; ++w) s += sh[w][k];
      out[k] = s;
    }
  }
}

// ---------------------------------------------------------------------------
// integrator stage 1 -- src/md_simulator.cpp:640-656 (velocity Verlet) and
// :748-837 (Langevin first half); NaN check; half-skin test per replica
// ---------------------------------------------------------------------------
__device__ inline void update_rel(const Dev &d, const RepBox &rb, int i, const dbl4 &x) {
  const int c = d.cell_of[i] - rb.cell_off;
  const int cx = c % rb.nc[0], cy = (c / rb.nc[0]) % rb.nc[1], cz = c / (rb.nc[0] * rb.nc[1]);
  float4 r;
  r.x = (float)(x.x - (rb.lo[0] + cx * rb.w[0]));
  r.y = (float)(x.y - (rb.lo[1] + cy * rb.w[1]));
  r.z = (float)(x.z - (rb.lo[2] + cz * rb.w[2]));
  r.w = __int_as_float(type_of(x.w));
  d.rel[i] = r;
}

// Velocity-Verlet drift (src/md_simulator.cpp:640-656) with the NaN check of the
// acceleration and the half-skin test; the pair kernel fuses the same update into
// the step before when it can (FUSE_VV), so this kernel runs at the start of a chunk.
template <bool MIXED>
__global__ void __launch_bounds__(256) k_drift_vv(Dev d, Box b, StepConsts sc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= sc.n || halted(d)) return;
  const int rep = rep_of_slot(b, i);
  if (rep < 0) return;  // padding slot
  dbl4 x = d.pos[i];
  const dbl4 v = d.vel[i], a = d.acc[i];
  nan_check(d, i, a);
  drift_vv<MIXED>(x, v, a, sc);
  d.pos[i] = x;  // acc stays: the pair kernel's kick reads it as a_old
  if (MIXED) mixed_track(d, b, rep, i, x, d.rel);
  else half_skin_test(d, b, rep, i, x);
}

// Leap-frog first half (src/md_simulator.cpp:890-905): v += (0.5 dt) a ; r += dt v.
// The closing half, v += (0.5 dt) a(t + dt), is the velocity-Verlet kick of the pair
// kernel with a_old = 0: v + (a + 0)(0.5 dt) rounds exactly as v + (0.5 dt) a.
template <bool MIXED>
__global__ void __launch_bounds__(256) k_drift_lf(Dev d, Box b, StepConsts sc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= sc.n || halted(d)) return;
  const int rep = rep_of_slot(b, i);
  if (rep < 0) return;  // padding slot
  dbl4 x = d.pos[i], v = d.vel[i];
  const dbl4 a = d.acc[i];
  nan_check(d, i, a);
  drift_lf<MIXED>(x, v, a, sc);
  d.pos[i] = x;
  d.vel[i] = v;
  d.acc[i] = make_dbl4(0.0, 0.0, 0.0, 0.0);  // a_old = 0 for the kick
  if (MIXED) mixed_track(d, b, rep, i, x, d.rel);
  else half_skin_test(d, b, rep, i, x);
}

// Langevin position update r += v*c (src/md_simulator.cpp:822-827) with the
// half-skin tracking; with THERMO the temperature sums of the velocities first.
template <bool MIXED, bool THERMO>
__device__ __forceinline__ void lang_position(const Dev &d, const Box &b, const StepConsts &sc, int rep, int i, dbl4 x,
                                              const dbl4 &v, double (&part)[4]) {
  if (THERMO) {
    const double m = d.tab->mass[type_of(x.w)];
    part[0] = m * (v.x * v.x + v.y * v.y + v.z * v.z);
    part[1] = m * v.x; part[2] = m * v.y; part[3] = m * v.z;
  }
  lang_move<MIXED>(x, v, sc);
  d.pos[i] = x;
  if (MIXED) mixed_track(d, b, rep, i, x, d.rel);
  else half_skin_test(d, b, rep, i, x);
}

// Langevin first half (src/md_simulator.cpp:748-837):
//   v += (a*0.5)*dt + eta*b ; [temperature here] ; r += v*c
// POS false: the velocity half only; constraint::Nve then acts on the mid-step
// velocities (:784-791) and k_lang_pos takes the temperature and moves the atoms.
template <bool MIXED, bool THERMO, bool POS>
__global__ void __launch_bounds__(256) k_lang_a(Dev d, Box b, StepConsts sc, int k_in_chunk) {
  if (halted(d)) return;  // the same value for every block: no block reaches the reduction alone
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double part[4] = {0.0, 0.0, 0.0, 0.0};
  const int rep = i < sc.n ? rep_of_slot(b, i) : -1;
  if (rep >= 0) {
    dbl4 x = d.pos[i], v = d.vel[i];
    const dbl4 a = d.acc[i];
    nan_check(d, i, a);
    double e0 = 0.0, e1 = 0.0, e2 = 0.0;
    if (!sc.noise_off) {
      const long long step = *d.step_base + k_in_chunk;
      // replica r draws the noise stream of seed + r with its local ids
      if (MIXED) langevin_eta_f(sc.seed + rep, step, d.id[i], e0, e1, e2);
      else langevin_eta(sc.seed + rep, step, d.id[i], e0, e1, e2);
    }
    lang_half<MIXED>(v, a, e0, e1, e2, sc);
    d.vel[i] = v;
    if (POS) lang_position<MIXED, THERMO>(d, b, sc, rep, i, x, v, part);
  }
  if (POS && THERMO) block_sum_store<4>(part, &d.partials_ke[(size_t)blockIdx.x * 4]);
}

template <bool MIXED, bool THERMO>
__global__ void __launch_bounds__(256) k_lang_pos(Dev d, Box b, StepConsts sc) {
  if (halted(d)) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double part[4] = {0.0, 0.0, 0.0, 0.0};
  const int rep = i < sc.n ? rep_of_slot(b, i) : -1;
  if (rep >= 0) lang_position<MIXED, THERMO>(d, b, sc, rep, i, d.pos[i], d.vel[i], part);
  if (THERMO) block_sum_store<4>(part, &d.partials_ke[(size_t)blockIdx.x * 4]);
}

// ---------------------------------------------------------------------------
// list rebuild of the flagged replicas: wrap + bin -> per-replica scan ->
// scatter -> per-cell sort -> gather -> build
// (Neighborlist::update_cell_list + update_verlet_list_from_cell_list,
//  src/neighborlist.cpp:422-455, 496-553; Domain::fix_position, src/domain.cpp:443-493)
// ---------------------------------------------------------------------------
// a rebuild pass builds the replicas whose half-skin test fired (all when forced);
// nothing after a halt
__device__ inline bool rebuild_on(const Dev &d, const Box &b, int rep, int forced) {
  return !halted(d) && (forced || b.rep_flag[rep] != 0);
}

// Domain::fix_position's single-image test per axis (src/domain.cpp:443-493):
// -1 below the lower face (x += L), +1 above the upper face (x -= L), else 0
__device__ inline int3 wrap_shift(const RepBox &rb, const dbl4 &p) {
  return make_int3(p.x < rb.lo[0] ? -1 : (p.x > rb.hi[0] ? 1 : 0), p.y < rb.lo[1] ? -1 : (p.y > rb.hi[1] ? 1 : 0),
                   p.z < rb.lo[2] ? -1 : (p.z > rb.hi[2] ? 1 : 0));
}

__global__ void __launch_bounds__(256) k_bin(Dev d, Box b, int forced) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) d.flags[F_MAXNB] = 0;
  int rep = i < b.nslot ? rep_of_slot(b, i) : -1;
  const bool act = rep >= 0 && rebuild_on(d, b, rep, forced);
  int c = 0;
  if (act) {
    const RepBox &rb = repbox(b, rep);
    dbl4 p = d.pos[i];
    // single-image wrap exactly as Domain::fix_position, counting the crossings
    // (+1 through the upper face) as exchange_owned adds them to msd_domain_cross
    const int3 w = wrap_shift(rb, p);
    if (w.x | w.y | w.z) {  // the few atoms that left the box
      if (w.x) p.x += w.x > 0 ? -rb.L[0] : rb.L[0];
      if (w.y) p.y += w.y > 0 ? -rb.L[1] : rb.L[1];
      if (w.z) p.z += w.z > 0 ? -rb.L[2] : rb.L[2];
      d.pos[i] = p;
      if (d.img) {
        int4 m = d.img[i];
        m.x += w.x; m.y += w.y; m.z += w.z;
        d.img[i] = m;
      }
    }
    const double ux = (p.x - rb.lo[0]) * rb.inv_w[0], uy = (p.y - rb.lo[1]) * rb.inv_w[1],
                 uz = (p.z - rb.lo[2]) * rb.inv_w[2];
    int cx = (int)floor(ux), cy = (int)floor(uy), cz = (int)floor(uz);
    cx = min(max(cx, 0), rb.nc[0] - 1);
    cy = min(max(cy, 0), rb.nc[1] - 1);
    cz = min(max(cz, 0), rb.nc[2] - 1);
    c = rb.cell_off + cx + rb.nc[0] * (cy + rb.nc[1] * cz);
    d.atom_cell[i] = c;
    // order inside the cell: the Morton index of the atom's 4x4x4 sub-cell, then its id,
    // so that consecutive slots (a warp's lanes) sit close together and their neighbour
    // lists run through the same candidates
    const int sx = min(max((int)((ux - cx) * 4.0), 0), 3), sy = min(max((int)((uy - cy) * 4.0), 0), 3),
              sz = min(max((int)((uz - cz) * 4.0), 0), 3);
    const uint32_t morton = (sx & 1) | ((sy & 1) << 1) | ((sz & 1) << 2) | ((sx & 2) << 2) | ((sy & 2) << 3) |
                            ((sz & 2) << 4);
    d.skey[i] = ((uint64_t)morton << 32) | d.id[i];
  }
  // warp-aggregated counting: one atomic per distinct cell in the warp
  const unsigned m = __ballot_sync(FULL_MASK, act);
  if (act) {
    const unsigned peers = __match_any_sync(m, c);
    if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&d.cell_count[c], __popc(peers));
  }
}

// Exclusive scan of each replica's cell counts, starting at the replica's first
// slot; the padding cell counts the replica's padding slots.  Block rep*P + p owns
// slice p of the replica's m counts (scan_slice(m, P, p); P > 1 only for a single
// system, whose slices start from the sums k_scan_part left in scan_part).
// Warp w owns the contiguous run [w*seg, (w+1)*seg) of its slice and walks it 32
// counts at a time with coalesced loads: a first pass sums the run, one scan of the
// 32 warp sums gives every run its start, and a second pass scans the run (warp
// shuffles, carry from lane 31) and writes the starts.  Zeroes the counts and
// cursors it read.
__device__ inline int2 scan_slice(int m, int P, int p) {
  const int len = ((m + P - 1) / P + 31) & ~31;
  const int s0 = min(m, p * len);
  return make_int2(s0, min(m, s0 + len));
}

__device__ inline int scan_count(const Dev &d, const RepBox &rb, int m, int k) {
  return k == m - 1 ? rb.pad : d.cell_count[rb.cell_off + k];
}

// single system: the sum of each slice's counts (first level of the scan)
__global__ void __launch_bounds__(1024) k_scan_part(Dev d, Box b, int forced) {
  if (!rebuild_on(d, b, 0, forced)) return;
  const RepBox &rb = repbox(b, 0);
  const int m = rb.ncell + 1;
  const int2 sl = scan_slice(m, gridDim.x, blockIdx.x);
  int v = 0;
  for (int k = sl.x + (int)threadIdx.x; k < sl.y; k += blockDim.x) v += scan_count(d, rb, m, k);
  __shared__ int warp_tot[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
  if (lane == 0) warp_tot[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
    if (lane == 0) d.scan_part[blockIdx.x] = v;
  }
}

__global__ void __launch_bounds__(1024) k_scan_rep(Dev d, Box b, int forced, int P) {
  const int rep = blockIdx.x / P, p = blockIdx.x - rep * P;
  if (!rebuild_on(d, b, rep, forced)) return;
  const RepBox &rb = repbox(b, rep);
  const int m = rb.ncell + 1, off = rb.cell_off;
  const int2 sl = scan_slice(m, P, p);
  __shared__ int warp_tot[32];
  __shared__ int slice_base;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  if (wid == 0) {  // counts before this slice: the first-level sums of slices 0 .. p-1
    int v = 0;
    for (int q = lane; q < p; q += 32) v += d.scan_part[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
    if (lane == 0) slice_base = v;
  }
  const int seg = ((sl.y - sl.x + 31) / 32 + 31) & ~31;  // counts per warp, a multiple of 32
  const int k0 = min(sl.y, sl.x + wid * seg), k1 = min(sl.y, k0 + seg);
  auto count = [&](int k) { return k < k1 ? scan_count(d, rb, m, k) : 0; };
  int s = 0;
#pragma unroll 4
  for (int k = k0 + lane; k < k1; k += 32) s += count(k);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL_MASK, s, o);
  if (lane == 0) warp_tot[wid] = s;
  __syncthreads();
  if (wid == 0) {
    int wv = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(FULL_MASK, wv, o);
      if (lane >= o) wv += y;
    }
    warp_tot[lane] = wv;  // inclusive
  }
  __syncthreads();
  int carry = rb.slot_off + slice_base + (wid ? warp_tot[wid - 1] : 0);
  for (int base = k0; base < k1; base += 32) {
    const int k = base + lane;
    const int v = count(k);
    int inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(FULL_MASK, inc, o);
      if (lane >= o) inc += y;
    }
    if (k < k1) {
      d.cell_start[off + k] = carry + inc - v;
      d.cell_count[off + k] = 0;
      d.cell_cursor[off + k] = 0;
    }
    carry += __shfl_sync(FULL_MASK, inc, 31);
  }
}

__global__ void __launch_bounds__(256) k_scatter(Dev d, Box b, int forced) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.nslot) return;
  const int rep = rep_of_slot(b, i);
  if (rep < 0 || !rebuild_on(d, b, rep, forced)) return;
  const int c = d.atom_cell[i];
  d.perm_tmp[d.cell_start[c] + atomicAdd(&d.cell_cursor[c], 1)] = i;
}

// one warp per cell: order the cell's atoms by their sort key (sub-cell, then host
// index: deterministic lists); cells of up to 32 atoms rank in registers with warp
// shuffles
__global__ void __launch_bounds__(256) k_cell_sort(Dev d, Box b, int forced) {
  const int cell = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (cell >= b.ncell_all) return;
  const int rep = rep_of_cell(b, cell);
  if (rep < 0 || !rebuild_on(d, b, rep, forced)) return;
  const int s = d.cell_start[cell], e = d.cell_start[cell + 1], n = e - s;
  if (n <= 32) {
    const int ia = lane < n ? d.perm_tmp[s + lane] : 0;
    const uint64_t ka = lane < n ? d.skey[ia] : ~0ull;
    int rank = 0;
    for (int q = 0; q < n; ++q) rank += __shfl_sync(FULL_MASK, ka, q) < ka;
    if (lane < n) d.perm[s + rank] = ia;
    return;
  }
  for (int a = lane; a < n; a += 32) {
    const int ia = d.perm_tmp[s + a];
    const uint64_t ka = d.skey[ia];
    int rank = 0;
    for (int q = 0; q < n; ++q) rank += d.skey[d.perm_tmp[s + q]] < ka;
    d.perm[s + rank] = ia;
  }
}

__global__ void __launch_bounds__(256) k_copy_state(Dev d, Box b, int forced) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.nslot) return;
  const int rep = rep_of_slot(b, i);
  if (rep < 0 || !rebuild_on(d, b, rep, forced)) return;
  d.t_pos[i] = d.pos[i];
  d.t_vel[i] = d.vel[i];
  d.t_acc[i] = d.acc[i];  // a(t): the next kick reads it as a_old
  d.t_type[i] = d.type[i];
  d.t_id[i] = d.id[i];
  if (d.img) d.t_img[i] = d.img[i];
  if (d.mol) d.t_mol[i] = d.mol[i];
  d.perm_tmp[i] = d.atom_cell[i];  // cell of old slot i (perm_tmp is free again)
}

__global__ void __launch_bounds__(256) k_gather(Dev d, Box b, int forced) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= b.nslot) return;
  const int rep = rep_of_slot(b, k);
  if (rep < 0 || !rebuild_on(d, b, rep, forced)) return;
  const int o = d.perm[k];
  const dbl4 x = d.t_pos[o];
  d.pos[k] = x;
  d.pos_ref[k] = x;
  d.vel[k] = d.t_vel[o];
  d.acc[k] = d.t_acc[o];
  d.type[k] = d.t_type[o];
  d.id[k] = d.t_id[o];
  if (d.img) d.img[k] = d.t_img[o];
  if (d.mol) d.mol[k] = d.t_mol[o];
  d.cell_of[k] = d.perm_tmp[o];
  update_rel(d, repbox(b, rep), k, x);
  d.rel_ref[k] = d.rel[k];
}

// Verlet-list build over the 27-cell stencil with periodic image shifts.
// Predicate: r^2 < cutoff_extra^2 evaluated in FP64 exactly as the reference
// evaluates it for a ghost image (image = x_j + s*L, then minus x_i, squares
// summed x, y, z; no FMA contraction), pre-screened in FP32 on cell-relative
// coordinates: only candidates inside a narrow band around the cutoff take
// the FP64 path.  mode 0 stores image codes (FP64 force), mode 1 cell-offset
// codes (mixed force).
__device__ __noinline__ bool exact_pair(const Dev &d, const RepBox &rb, double ce2, int i, int j, int img) {
  const dbl4 xi = d.pos[i], xj = d.pos[j];
  const double shx = (img % 3 - 1) * rb.L[0], shy = ((img / 3) % 3 - 1) * rb.L[1], shz = (img / 9 - 1) * rb.L[2];
  const double ddx = __dsub_rn(__dadd_rn(xj.x, shx), xi.x);
  const double ddy = __dsub_rn(__dadd_rn(xj.y, shy), xi.y);
  const double ddz = __dsub_rn(__dadd_rn(xj.z, shz), xi.z);
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)), __dmul_rn(ddz, ddz));
  return r2 < ce2;
}

// Home groups.  A warp takes a window of 32 consecutive slots; the window's atoms
// that lie in one x-row of search cells, within GROUP_SPAN + 1 consecutive cells of
// it, form a group (a window that crosses the end of a row, or a sparse row, takes
// two or more groups in turn).  Slots are sorted by cell, so a group is 32 (or
// fewer) atoms from 1-3 neighbouring cells.  Its candidates are the atoms of the
// cells cx_first - 1 .. cx_last + 1 of the 3 x 3 neighbouring rows, taken row by row
// (dz, then dy, then x, slot order inside a cell), and of those only the ones within
// the list cutoff (plus the FP32 band) of the group's bounding box are staged: ~540
// staged candidates per 32 atoms of the 1M-atom fluid, against 27 cells x 19 atoms
// = 516 per 19-atom cell when a warp took one cell.  Every atom's row keeps the
// stencil order k = (dx+1) + 3(dy+1) + 9(dz+1), slot order inside a cell, so the
// lists do not depend on how slots fall into windows.
//
// Staging: candidates u and u+1 (u even) interleaved as {x_u, x_u+1, y_u, y_u+1}
// and {z_u, z_u+1} in the warp's slice of shared memory (coordinates relative to
// the origin of the group's first cell), the words (j | code) in an array of their
// own, plus one byte per candidate: its cell's x index in the group's window of
// cells and its row (dy, dz).  The sweep takes 32 candidates at a time, two per
// packed FP32x2 distance evaluation: every pair of candidates is two shared-memory
// broadcasts tested by all group atoms, the results collect in a hit and a band bit
// mask per lane (one warp vote per 32 candidates for the rare exact FP64 test), and
// only then are the hits (~15% of the staged candidates) written, in candidate order.
constexpr int BUILD_WARPS = 8;    // warps per block
constexpr int BUILD_STAGE = 256;  // staged candidates per warp and pass (4 KiB + 256 B)
constexpr int GROUP_SPAN = 5;     // a group spans at most 6 cells: x index + 8 row < 256

// q_u, q_u+1 = |c - r|^2 of two candidates with packed FP32x2 arithmetic (sm_100+):
// (cx - rx)^2, then + (cy - ry)^2, then + (cz - rz)^2, each rounded once
__device__ __forceinline__ void dist2_pair(const float4 &xy, const float2 &z, unsigned long long rxx,
                                           unsigned long long ryy, unsigned long long rzz, float &q0, float &q1) {
  asm("{\n\t.reg .b64 c, dd, q;\n\t"
      "mov.b64 c, {%2, %3};\n\tsub.rn.f32x2 dd, c, %8;\n\tmul.rn.f32x2 q, dd, dd;\n\t"
      "mov.b64 c, {%4, %5};\n\tsub.rn.f32x2 dd, c, %9;\n\tfma.rn.f32x2 q, dd, dd, q;\n\t"
      "mov.b64 c, {%6, %7};\n\tsub.rn.f32x2 dd, c, %10;\n\tfma.rn.f32x2 q, dd, dd, q;\n\t"
      "mov.b64 {%0, %1}, q;\n\t}"
      : "=f"(q0), "=f"(q1)
      : "f"(xy.x), "f"(xy.y), "f"(xy.z), "f"(xy.w), "f"(z.x), "f"(z.y), "l"(rxx), "l"(ryy), "l"(rzz));
}

__device__ __forceinline__ unsigned long long pack2(float v) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %1};" : "=l"(r) : "f"(v));
  return r;
}

// The lane's side of a group: its atom, where it sits in the group, its row.
struct BuildLane {
  int i;              // slot (valid when `me`)
  bool me;            // member of the current group
  int ci;             // x cell index within the group (0 .. span)
  int cx, cy, cz;     // cell of the atom
  int mol;            // molecule index (ignore_intra_molecule)
  unsigned long long rxx, ryy, rzz;  // the atom's coordinates in the group frame, packed twice
  float hi;           // upper end of the FP32 band (-1 for non-members: they never hit)
  uint32_t *row;      // the atom's list row
  int cnt;            // list words the atom has so far
  const int *selfpos; // shared: per lane, where its own atom sits in the current stage (-1: not in it)
};

// Sweep of nst staged candidates against every member of the group (see above).
// Staged words carry j and a code: the image code (MODE 0), or (MODE 1) the cell's
// x index in the group's window of cells plus 3 x its row, from which a member
// subtracts its own x index to get the stencil index of j's cell relative to its own.
template <int MODE>
__device__ __forceinline__ void build_sweep(const Dev &d, const Box &b, const RepBox &rb, int nst,
                                            const float4 *sxy, const float2 *sz, const uint32_t *sw,
                                            const uint8_t *su, BuildLane &L, int cshift, bool by_mol) {
  const int lane = threadIdx.x & 31;
  float *pxy = const_cast<float *>(reinterpret_cast<const float *>(sxy));
  float *pz = const_cast<float *>(reinterpret_cast<const float *>(sz));
  const int npad32 = (nst + 31) & ~31;
  for (int t = nst + lane; t < npad32; t += 32) {  // far-away padding up to a whole 32
    const int e = (t >> 1) * 4 + (t & 1);
    pxy[e] = 1e18f;
    pxy[e + 2] = 1e18f;
    pz[t] = 1e18f;
    const_cast<uint32_t *>(sw)[t] = 0u;
  }
  __syncwarp();
  const float lo = b.ce2_lo;
  const int cap = d.cap;
  const int self = L.selfpos[lane];
  const uint32_t ci_code = (uint32_t)L.ci << CODE_SHIFT;
  for (int t0 = 0; t0 < npad32; t0 += 32) {
    // phase 1: bits of the sure hits (q < ce2_lo) and of everything up to ce2_hi
    uint32_t hm = 0u, am = 0u;
#pragma unroll
    for (int u = 0; u < 32; u += 2) {
      const int pr = (t0 + u) >> 1;
      const float4 xy = sxy[pr];  // broadcast
      const float2 z = sz[pr];    // broadcast
      float q0, q1;
      dist2_pair(xy, z, L.rxx, L.ryy, L.rzz, q0, q1);
      if (q0 < lo) hm |= 1u << u;
      if (q0 <= L.hi) am |= 1u << u;
      if (q1 < lo) hm |= 2u << u;
      if (q1 <= L.hi) am |= 2u << u;
    }
    const int ts = self - t0;  // the atom itself is no candidate
    if (ts >= 0 && ts < 32) am &= ~(1u << ts);
    hm &= am;
    uint32_t bm = am & ~hm;  // the band
    const uint32_t *swc = sw + t0;
    if (__any_sync(FULL_MASK, bm != 0u)) {  // rare: the exact FP64 predicate
      while (bm) {
        const int u = __ffs(bm) - 1;
        bm &= bm - 1u;
        const int t = t0 + u;
        const uint32_t w = swc[u];
        const int j = (int)(w & IDX_MASK);
        int img = (int)(w >> CODE_SHIFT);
        if (MODE != 0) {  // the image from the candidate cell's unwrapped index
          const int s = su[t], r = s >> 3;
          const int nx = L.cx + (s & 7) - 1 - L.ci, ny = L.cy + r % 3 - 1, nz = L.cz + r / 3 - 1;
          img = image_code(nx < 0 ? -1 : (nx >= rb.nc[0] ? 1 : 0), ny < 0 ? -1 : (ny >= rb.nc[1] ? 1 : 0),
                           nz < 0 ? -1 : (nz >= rb.nc[2] ? 1 : 0));
        }
        if (exact_pair(d, rb, b.ce2, L.i, j, img)) hm |= 1u << u;
      }
    }
    // phase 2: the hits, in candidate order (with ignore_intra_molecule none of the
    // atom's own molecule, as Lj::calculate_acceleration skips them, src/force/lj.cpp:446)
    while (hm) {
      const int u = __ffs(hm) - 1;
      hm &= hm - 1u;
      uint32_t w = swc[u];
      if (by_mol && d.mol[w & IDX_MASK] == L.mol) continue;
      if (MODE != 0) w -= ci_code;  // stencil index of j's cell relative to the atom's
      if (L.cnt < cap) L.row[((L.cnt >> 2) << cshift) + (L.cnt & 3)] = w;
      ++L.cnt;
    }
  }
  __syncwarp();  // the stage is refilled next
}

__device__ inline float warp_minf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(FULL_MASK, v, o));
  return v;
}
__device__ inline float warp_maxf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(FULL_MASK, v, o));
  return v;
}

template <int MODE>
__global__ void __launch_bounds__(BUILD_WARPS * 32, 4) k_build_group(Dev d, Box b, int forced) {
  __shared__ float4 sxy_all[BUILD_WARPS][BUILD_STAGE / 2];
  __shared__ float2 sz_all[BUILD_WARPS][BUILD_STAGE / 2];
  __shared__ uint32_t sw_all[BUILD_WARPS][BUILD_STAGE];
  __shared__ uint8_t su_all[BUILD_WARPS][BUILD_STAGE];
  __shared__ int selfpos_all[BUILD_WARPS][32];
  const int lane = threadIdx.x & 31;
  // pair p = candidates 2p, 2p+1: sxy[p] = {x, x', y, y'}, sz[p] = {z, z'}; sw[t] = word of t
  float4 *sxy = sxy_all[threadIdx.x >> 5];
  float2 *sz = sz_all[threadIdx.x >> 5];
  uint32_t *sw = sw_all[threadIdx.x >> 5];
  float *fxy = reinterpret_cast<float *>(sxy), *fz = reinterpret_cast<float *>(sz);
  uint8_t *su = su_all[threadIdx.x >> 5];
  const bool by_mol = d.mol != nullptr;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  const int cshift = 7 - log2_pow2(d.tpa);  // chunk stride 4A words = 2^(log2 A + 2)
  const unsigned lt_mask = (1u << lane) - 1u;
  const int nwin = (b.nslot + 31) >> 5;
  int wmax = 0;
  for (int win = gw; win < nwin; win += nw) {
    BuildLane L;
    L.i = (win << 5) + lane;
    const int rep = L.i < b.nslot ? rep_of_slot(b, L.i) : -1;
    const bool act = rep >= 0 && rebuild_on(d, b, rep, forced);
    int rowkey = -1;  // global index of the first cell of the atom's row: one value per (replica, row)
    float4 ri = make_float4(0.f, 0.f, 0.f, 0.f);
    L.cx = L.cy = L.cz = 0;
    L.mol = 0;
    if (act) {
      const RepBox &rb = repbox(b, rep);
      const int c = d.cell_of[L.i], lc = c - rb.cell_off;
      L.cx = lc % rb.nc[0];
      L.cy = (lc / rb.nc[0]) % rb.nc[1];
      L.cz = lc / (rb.nc[0] * rb.nc[1]);
      rowkey = c - L.cx;
      ri = d.rel[L.i];
      if (d.mol) L.mol = d.mol[L.i];
    }
    L.row = d.nbr + nbr_block_base(act ? L.i : 0, d.cap, d.tpa);
    int *selfpos = selfpos_all[threadIdx.x >> 5];
    L.selfpos = selfpos;
    const int win0 = win << 5;
    unsigned pending = __ballot_sync(FULL_MASK, act);
    while (pending) {
      const int leader = __ffs(pending) - 1;
      const int rk = __shfl_sync(FULL_MASK, rowkey, leader);
      const int cx0 = __shfl_sync(FULL_MASK, L.cx, leader);  // slots sort by cell: the leader's is the lowest
      const int grep = __shfl_sync(FULL_MASK, rep, leader);
      const unsigned mem = __ballot_sync(FULL_MASK, ((pending >> lane) & 1u) && rowkey == rk && L.cx - cx0 <= GROUP_SPAN);
      pending &= ~mem;
      L.me = (mem >> lane) & 1u;
      const RepBox &rb = repbox(b, grep);
      const int span = __reduce_max_sync(FULL_MASK, L.me ? L.cx - cx0 : 0);
      L.ci = L.me ? L.cx - cx0 : 0;
      const int cy = __shfl_sync(FULL_MASK, L.cy, leader), cz = __shfl_sync(FULL_MASK, L.cz, leader);
      // the atom in the group frame (origin: the group's first cell), and the group's box
      const float gx = ri.x + (float)L.ci * rb.wf[0], gy = ri.y, gz = ri.z;
      const float bxl = warp_minf(L.me ? gx : 1e30f), bxh = warp_maxf(L.me ? gx : -1e30f);
      const float byl = warp_minf(L.me ? gy : 1e30f), byh = warp_maxf(L.me ? gy : -1e30f);
      const float bzl = warp_minf(L.me ? gz : 1e30f), bzh = warp_maxf(L.me ? gz : -1e30f);
      L.rxx = pack2(gx);
      L.ryy = pack2(gy);
      L.rzz = pack2(gz);
      L.hi = L.me ? b.ce2_hi : -1.0f;
      L.cnt = 0;
      // candidate cells q = r * nu + u: row r = (dy+1) + 3 (dz+1), x cell cx0 - 1 + u
      const int nu = span + 3, ncand = 9 * nu;
      int nst = 0;
      selfpos[lane] = -1;
      __syncwarp();
      for (int q0 = 0; q0 < ncand; q0 += 32) {
        // lane q - q0: the candidate cell's first slot, count, image code, origin offset
        int kb = 0, kn = 0, ks = 0, kimg = 0;
        uint32_t kcode = 0u;
        float kox = 0.f, koy = 0.f, koz = 0.f;
        const int q = q0 + lane;
        if (q < ncand) {
          const int r = q / nu, u = q - r * nu;
          const int dy = r % 3 - 1, dz = r / 3 - 1;
          int nx = cx0 - 1 + u, ny = cy + dy, nz = cz + dz, sx = 0, sy = 0, sz = 0;
          if (nx < 0) { nx += rb.nc[0]; sx = -1; } else if (nx >= rb.nc[0]) { nx -= rb.nc[0]; sx = 1; }
          if (ny < 0) { ny += rb.nc[1]; sy = -1; } else if (ny >= rb.nc[1]) { ny -= rb.nc[1]; sy = 1; }
          if (nz < 0) { nz += rb.nc[2]; sz = -1; } else if (nz >= rb.nc[2]) { nz -= rb.nc[2]; sz = 1; }
          const int c2 = rb.cell_off + nx + rb.nc[0] * (ny + rb.nc[1] * nz);
          kb = d.cell_start[c2];
          kn = d.cell_start[c2 + 1] - kb;
          // mode 0: the image code; mode 1: x index + 3 x row (<= 7 + 24), from which a
          // member's stencil index follows by subtracting its own x index
          kimg = image_code(sx, sy, sz);
          kcode = (uint32_t)(MODE == 0 ? kimg : u + 3 * r) << CODE_SHIFT;
          ks = u | (r << 3);
          kox = (float)(u - 1) * rb.wf[0];
          koy = (float)dy * rb.wf[1];
          koz = (float)dz * rb.wf[2];
        }
        const int kend = min(32, ncand - q0);
        for (int k = 0; k < kend; ++k) {
          const int cn = __shfl_sync(FULL_MASK, kn, k);
          if (cn == 0) continue;
          const int jb = __shfl_sync(FULL_MASK, kb, k);
          const uint32_t code = __shfl_sync(FULL_MASK, kcode, k);
          const uint8_t sbyte = (uint8_t)__shfl_sync(FULL_MASK, ks, k);
          const bool zero_img = __shfl_sync(FULL_MASK, kimg, k) == CODE_ZERO;
          const float ox = __shfl_sync(FULL_MASK, kox, k), oy = __shfl_sync(FULL_MASK, koy, k),
                      oz = __shfl_sync(FULL_MASK, koz, k);
          for (int t0 = 0; t0 < cn; t0 += 32) {
            const int t = t0 + lane;
            bool keep = false;
            float X = 0.f, Y = 0.f, Z = 0.f;
            if (t < cn) {
              const float4 rj = __ldg(&d.rel[jb + t]);
              X = rj.x + ox;
              Y = rj.y + oy;
              Z = rj.z + oz;
              // squared distance to the group's box; within the band's upper end: staged
              const float ex = fmaxf(fmaxf(bxl - X, X - bxh), 0.f), ey = fmaxf(fmaxf(byl - Y, Y - byh), 0.f),
                          ez = fmaxf(fmaxf(bzl - Z, Z - bzh), 0.f);
              keep = fmaf(ez, ez, fmaf(ey, ey, ex * ex)) <= b.ce2_hi;
            }
            const unsigned km = __ballot_sync(FULL_MASK, keep);
            if (keep) {
              const int s = nst + __popc(km & lt_mask);
              const int e = (s >> 1) * 4 + (s & 1);
              fxy[e] = X;
              fxy[e + 2] = Y;
              fz[s] = Z;
              sw[s] = (uint32_t)(jb + t) | code;
              su[s] = sbyte;
              // a window atom at its own cell and zero image: that lane's self position
              const unsigned l = (unsigned)(jb + t - win0);
              if (zero_img && l < 32u) selfpos[l] = s;
            }
            nst += __popc(km);
            if (nst > BUILD_STAGE - 32) {
              __syncwarp();
              build_sweep<MODE>(d, b, rb, nst, sxy, sz, sw, su, L, cshift, by_mol);
              selfpos[lane] = -1;
              __syncwarp();
              nst = 0;
            }
          }
        }
      }
      if (nst > 0) {
        __syncwarp();
        build_sweep<MODE>(d, b, rb, nst, sxy, sz, sw, su, L, cshift, by_mol);
      }
      if (L.me) {
        d.nnbr[L.i] = min(L.cnt, d.cap);
        if (L.cnt > d.cap) atomicMax(&d.flags[F_OVERFLOW], L.cnt);
        wmax = max(wmax, L.cnt);
      }
    }
  }
  // one atomic per warp for the largest list length (not one per atom)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(FULL_MASK, wmax, o));
  if (lane == 0 && wmax > 0) atomicMax(&d.flags[F_MAXNB], wmax);
}

// after the build: count the rebuilt replicas, clear their flags and the global one;
// a build that overflowed its rows halts the chunk (the host grows the list and
// completes the step)
__global__ void __launch_bounds__(256) k_finish_rebuild(Dev d, Box b, int forced) {
  if (halted(d)) return;
  __shared__ int total;
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  int n = 0;
  for (int r = threadIdx.x; r < b.nrep; r += blockDim.x) {
    n += (forced || b.rep_flag[r] != 0) ? 1 : 0;
    b.rep_flag[r] = 0;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(FULL_MASK, n, o);
  if ((threadIdx.x & 31) == 0 && n) atomicAdd_block(&total, n);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (total) {
      d.flags[F_REBUILDS] += total;
      d.flags[F_PASSES] += 1;
    }
    d.flags[F_REBUILD] = 0;
    if (d.flags[F_OVERFLOW]) d.flags[F_HALT] = 1;
  }
}

// Inside a captured step that starts with a drift kernel: a NaN the drift saw halts
// the chunk, and the half-skin flag becomes the value of the graph's conditional
// node that wraps the rebuild kernels (when the pair kernel drifted the step, its
// last block does both).
__global__ void k_set_rebuild_cond(Dev d, cudaGraphConditionalHandle h) {
  if (d.flags[F_NAN]) d.flags[F_HALT] = 1;
  cudaGraphSetConditional(h, (d.flags[F_REBUILD] != 0 && d.flags[F_HALT] == 0) ? 1u : 0u);
}

// the same NaN check for steps launched from the host (no conditional node)
__global__ void k_halt_check(Dev d) {
  if (d.flags[F_NAN]) d.flags[F_HALT] = 1;
}

// ---------------------------------------------------------------------------
// thermo: fold the per-block partials (fixed order) into KE, T, P, virial, PE
// (Atom_data::kinetic_energy_mpi_domain / finalize_temperature / finalize_pressure,
//  src/atom_data/kinetic_energy.cpp:26-134, 189-198, 238-303)
// thermo[] = {KE, T, P, virial, PE, sum m, -, -}
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_thermo_final(Dev d, ThermoCfg tc, int nb_ke, int nb_ev, int nb_ke_end,
                                                      int ring_slot) {
  if (halted(d)) return;  // every block alike: the ticket is not taken
  // level 1: block g folds partials g*256 + tid, stepping by the grid's threads (one
  // round of independent loads for up to 8192 partials)
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  double v[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = gt; k < nb_ke; k += gs)
    for (int q = 0; q < 4; ++q) v[q] += d.partials_ke[(size_t)k * 4 + q];
  const double *ev = d.partials_ev;
  for (int k = gt; k < nb_ev; k += gs) {
    v[4] += ev[(size_t)k * 2];
    v[5] += ev[(size_t)k * 2 + 1];
  }
  for (int k = gt; k < nb_ke_end; k += gs)
    for (int q = 0; q < 4; ++q) v[6 + q] += d.partials_ke_end[(size_t)k * 4 + q];
  __shared__ double out[10];
  __shared__ bool last;
  block_sum_store<10>(v, out);
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < 10; ++q) d.fold[blockIdx.x * 10 + q] = out[q];
    __threadfence();
    last = atomicAdd(d.fold_ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  // level 2, in the last block: the blocks' sums in block order.  All loads first
  // (L2-coherent, independent of one another), then the adds in block order: a
  // volatile load per add waited a full L2 round trip 32 times in a row
  if (threadIdx.x < 10) {
    __threadfence();
    double v[THERMO_FOLD_BLOCKS];
#pragma unroll
    for (int g = 0; g < THERMO_FOLD_BLOCKS; ++g) v[g] = __ldcg(&d.fold[g * 10 + threadIdx.x]);
    double s = 0.0;
#pragma unroll
    for (int g = 0; g < THERMO_FOLD_BLOCKS; ++g) s += v[g];
    out[threadIdx.x] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *d.fold_ticket = 0u;
    double res[5];
    const double P3[3] = {out[1], out[2], out[3]};
    // total mass is fixed at upload (thermo[5])
    thermo_finish(out[0], P3, d.thermo[5], out[4], out[5], tc.n, tc.n_r_df, tc.k_b, tc.volume, tc.langevin, res);
    if (nb_ke_end > 0) {  // KE as Atom_data::kinetic_energy() reads it after the step
      double e[5];
      const double Q3[3] = {out[7], out[8], out[9]};
      thermo_finish(out[6], Q3, d.thermo[5], 0.0, 0.0, tc.n, tc.n_r_df, tc.k_b, tc.volume, tc.langevin, e);
      res[0] = e[0];
    }
    for (int q = 0; q < 5; ++q) d.thermo[q] = res[q];
    if (ring_slot >= 0) {
      double *r = d.thermo_ring + (size_t)ring_slot * THERMO_REC;
      for (int q = 0; q < THERMO_REC; ++q) r[q] = res[q];
    }
  }
}

// Batches: one block per replica folds its slots in a fixed order.  ke: KE/T/P
// from the current velocities; ev: virial and PE from the per-slot sums the
// force kernel wrote (VV: P gets the virial term).  thermo_rep[r*8 + 0..5].
__global__ void __launch_bounds__(256) k_thermo_rep(Dev d, Box b, ThermoCfg tc, int ke, int ev) {
  if (halted(d)) return;
  const int rep = blockIdx.x;
  const RepBox &rb = repbox(b, rep);
  double v[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int i = rb.slot_off + threadIdx.x; i < rb.slot_off + rb.natoms; i += blockDim.x) {
    if (ke) {
      const dbl4 vv = d.vel[i];
      const double m = d.tab->mass[d.type[i]];
      v[0] += m * (vv.x * vv.x + vv.y * vv.y + vv.z * vv.z);
      v[1] += m * vv.x; v[2] += m * vv.y; v[3] += m * vv.z;
      v[4] += m;
    }
    if (ev) {
      const double2 e = d.ev_atom[i];
      v[5] += e.x;
      v[6] += e.y;
    }
  }
  __shared__ double out[7];
  block_sum_store<7>(v, out);
  __syncthreads();
  if (threadIdx.x == 0) {
    double *o = d.thermo_rep + (size_t)rep * 8;
    const double volume = rb.L[0] * rb.L[1] * rb.L[2];
    if (ke) {
      double res[5];
      const double P3[3] = {out[1], out[2], out[3]};
      thermo_finish(out[0], P3, out[4], 0.0, 0.0, rb.natoms, tc.n_r_df, tc.k_b, volume, 1, res);
      o[0] = res[0]; o[1] = res[1]; o[2] = res[2]; o[5] = out[4];
    }
    if (ev) {
      o[3] = 0.5 * out[5];
      o[4] = 0.5 * out[6];
      if (!tc.langevin) o[2] += o[3] / (3.0 * volume);
    }
  }
}

// end of a chunk: the step counter advances by the steps whose pair kernel ran; a
// halted chunk records how many that were (the host completes the failed step)
__global__ void k_advance_step(Dev d) {
  const int ok = d.flags[F_STEPS_OK];
  *d.step_base += ok;
  if (d.flags[F_HALT]) d.flags[F_HALT_STEP] += ok;
  d.flags[F_STEPS_OK] = 0;
}

// ---------------------------------------------------------------------------
// constraint::Nve (src/constraint/nve.cpp:132-184), single system: on steps whose
// index is a multiple of `step`, lambda = sqrt(target / KE) with KE the kinetic
// energy of Atom_data::kinetic_energy (centre-of-mass part removed for n_r_df
// 1..3), velocities scaled by lambda, then the temperature and pressure of the
// step follow the scaled velocities (finalize_temperature / finalize_pressure).
// ---------------------------------------------------------------------------
__device__ inline bool nve_applies(const Dev &d, const NveCfg &c, int k) {
  return !halted(d) && (*d.step_base + k) % c.step == 0;
}

__global__ void __launch_bounds__(256) k_nve_ke(Dev d, int n, NveCfg c, int k) {
  if (!nve_applies(d, c, k)) return;
  double part[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const dbl4 v = d.vel[i];
    const double m = d.tab->mass[d.type[i]];
    part[0] += m * (v.x * v.x + v.y * v.y + v.z * v.z);
    part[1] += m * v.x; part[2] += m * v.y; part[3] += m * v.z;
  }
  block_sum_store<4>(part, &d.nve_partials[(size_t)blockIdx.x * 4]);
}

__global__ void __launch_bounds__(256) k_nve_lambda(Dev d, ThermoCfg tc, NveCfg c, int k, int thermo, int ring_slot) {
  if (!nve_applies(d, c, k)) return;
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < NVE_BLOCKS; b += blockDim.x)
    for (int q = 0; q < 4; ++q) v[q] += d.nve_partials[(size_t)b * 4 + q];
  __shared__ double s[4];
  block_sum_store<4>(v, s);
  __syncthreads();
  if (threadIdx.x != 0) return;
  double ke2 = s[0];
  const double msum = d.thermo[5];
  if (tc.n_r_df >= 1 && tc.n_r_df <= 3 && msum > 0) ke2 -= (s[1] * s[1] + s[2] * s[2] + s[3] * s[3]) / msum;
  const double ke = 0.5 * ke2;
  const double dof = (double)(3 * tc.n - tc.n_r_df);  // Atom_data::degree_of_freedoms
  double lambda = 1.0;
  if (c.mode == CAVGPU_NVE_ENERGY_PER_DOF) lambda = sqrt(c.value * dof / ke);
  else if (c.mode == CAVGPU_NVE_ENERGY_TOT) lambda = sqrt(c.value / ke);
  else if (c.mode == CAVGPU_NVE_KBT) lambda = sqrt(dof * c.value * 0.5 / ke);
  else lambda = sqrt(dof * c.kb * c.value * 0.5 / ke);
  *d.nve_lambda = lambda;
  if (thermo) {  // the thermo point of this step: KE and T of the scaled velocities, P from them
    const double l2 = lambda * lambda;
    double *o = d.thermo;
    o[0] *= l2;
    o[1] *= l2;
    o[2] = ((double)tc.n * tc.k_b * o[1]) / tc.volume + (tc.langevin ? 0.0 : o[3]) / (3.0 * tc.volume);
    if (ring_slot >= 0)
      for (int q = 0; q < 3; ++q) d.thermo_ring[(size_t)ring_slot * THERMO_REC + q] = o[q];
  }
}

__global__ void __launch_bounds__(256) k_nve_scale(Dev d, int n, NveCfg c, int k) {
  if (!nve_applies(d, c, k)) return;
  const double lambda = *d.nve_lambda;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    dbl4 v = d.vel[i];
    v.x *= lambda; v.y *= lambda; v.z *= lambda;
    d.vel[i] = v;
  }
}

// ---------------------------------------------------------------------------
// parity exports
// ---------------------------------------------------------------------------
// what: 0 = positions (wrapped as Domain::fix_position), 1 = velocities, 2 = accelerations
__global__ void __launch_bounds__(256) k_to_host_order(Dev d, Box b, int what) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= b.nslot) return;
  const int rep = rep_of_slot(b, k);
  if (rep < 0) return;
  dbl4 v = what == 0 ? d.pos[k] : (what == 1 ? d.vel[k] : d.acc[k]);
  const RepBox &rb = repbox(b, rep);
  if (what == 0) {
    if (v.x < rb.lo[0]) v.x += rb.L[0]; else if (v.x > rb.hi[0]) v.x -= rb.L[0];
    if (v.y < rb.lo[1]) v.y += rb.L[1]; else if (v.y > rb.hi[1]) v.y -= rb.L[1];
    if (v.z < rb.lo[2]) v.z += rb.L[2]; else if (v.z > rb.hi[2]) v.z -= rb.L[2];
  }
  const size_t h = ((size_t)rb.id_off + d.id[k]) * 3;
  d.h3[h] = v.x; d.h3[h + 1] = v.y; d.h3[h + 2] = v.z;
}

// boundary crossings in host order: the stored counts plus the wrap the current
// position still owes (the reference wraps every step, the device at list builds)
__global__ void __launch_bounds__(256) k_images_to_host(Dev d, Box b) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= b.nslot) return;
  const int rep = rep_of_slot(b, k);
  if (rep < 0) return;
  const int3 w = wrap_shift(repbox(b, rep), d.pos[k]);
  const int4 m = d.img[k];
  const size_t h = ((size_t)repbox(b, rep).id_off + d.id[k]) * 3;
  d.hi3[h] = m.x + w.x; d.hi3[h + 1] = m.y + w.y; d.hi3[h + 2] = m.z + w.z;
}

// canonical rows (id_i, id_j, sx, sy, sz) of the current list (single system)
__global__ void __launch_bounds__(256) k_export_pairs(Dev d, Box b, int mode, int32_t *rows,
                                                      unsigned long long *counter, long long cap) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.nslot) return;
  const RepBox &rb = b.r0;
  const int ci = d.cell_of[i] - rb.cell_off;
  const int c3[3] = {ci % rb.nc[0], (ci / rb.nc[0]) % rb.nc[1], ci / (rb.nc[0] * rb.nc[1])};
  const int nn = d.nnbr[i];
  for (int k = 0; k < nn; ++k) {
    const uint32_t e = d.nbr[nbr_index(i, k, d.cap, d.tpa)];
    const int j = (int)(e & IDX_MASK), code = (int)(e >> CODE_SHIFT);
    int s[3] = {code % 3 - 1, (code / 3) % 3 - 1, code / 9 - 1};
    if (mode == 1)  // cell-offset code -> image shift
      for (int q = 0; q < 3; ++q) {
        const int c = c3[q] + s[q];
        s[q] = c < 0 ? -1 : (c >= rb.nc[q] ? 1 : 0);
      }
    const unsigned long long r = atomicAdd(counter, 1ull);
    if ((long long)r < cap) {
      int32_t *o = rows + r * 5;
      o[0] = (int32_t)d.id[i]; o[1] = (int32_t)d.id[j]; o[2] = s[0]; o[3] = s[1]; o[4] = s[2];
    }
  }
}

struct RefBins {
  double lo[3], inv;
  int nb[3];
};

__device__ inline void ref_bin(const RefBins &rb, double x, double y, double z, int32_t *o) {
  const double q[3] = {x, y, z};
  for (int a = 0; a < 3; ++a) {
    int v = (int)floor((q[a] - rb.lo[a]) * rb.inv);
    if (v < 0) v = 0;
    if (v >= rb.nb[a]) v = rb.nb[a] - 1;
    o[a] = v;
  }
}

// Neighborlist::binlist_index of each atom at its wrapped position (host order)
__global__ void __launch_bounds__(256) k_ref_bins(Dev d, int n, RefBins rb) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= n) return;
  ref_bin(rb, d.h3[3 * (size_t)h], d.h3[3 * (size_t)h + 1], d.h3[3 * (size_t)h + 2], &d.hi3[3 * (size_t)h]);
}

struct GhostCfg {
  double llow[3], lupp[3], L[3];
};

__device__ inline int ghost_vals(const GhostCfg &g, const double *q, int v[3]) {
  for (int a = 0; a < 3; ++a) v[a] = q[a] < g.llow[a] ? -1 : (q[a] > g.lupp[a] ? 1 : 0);
  const int nx = v[0] != 0, ny = v[1] != 0, nz = v[2] != 0;
  return nx + ny + nz + (nx & ny) + (nx & nz) + (ny & nz) + (nx & ny & nz);
}

__global__ void __launch_bounds__(256) k_ghost_count(Dev d, int n, GhostCfg g, int *counts) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= n) return;
  int v[3];
  counts[h] = ghost_vals(g, &d.h3[3 * (size_t)h], v);
}

// images in the order x, y, z, xy, xz, yz, xyz with coordinate pos - val*width
// (src/atom_data/exchange_ghost_single_md_domain.cpp:163-214)
__global__ void __launch_bounds__(256) k_ghost_emit(Dev d, int n, GhostCfg g, const int *starts, int32_t *src,
                                                    int32_t *shift3, double *pos3, int32_t *bins3, long long cap,
                                                    RefBins rb) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= n) return;
  const double *q = &d.h3[3 * (size_t)h];
  int v[3];
  ghost_vals(g, q, v);
  const double gx = q[0] - v[0] * g.L[0], gy = q[1] - v[1] * g.L[1], gz = q[2] - v[2] * g.L[2];
  const int combos[7][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
  long long o = starts[h];
  for (int c = 0; c < 7; ++c) {
    const int ux = combos[c][0], uy = combos[c][1], uz = combos[c][2];
    if ((ux && !v[0]) || (uy && !v[1]) || (uz && !v[2])) continue;
    if (o < cap) {
      const double p[3] = {ux ? gx : q[0], uy ? gy : q[1], uz ? gz : q[2]};
      src[o] = h;
      shift3[3 * o] = ux ? -v[0] : 0; shift3[3 * o + 1] = uy ? -v[1] : 0; shift3[3 * o + 2] = uz ? -v[2] : 0;
      pos3[3 * o] = p[0]; pos3[3 * o + 1] = p[1]; pos3[3 * o + 2] = p[2];
      ref_bin(rb, p[0], p[1], p[2], &bins3[3 * o]);
    }
    ++o;
  }
}

// exclusive scan of counts[0..m) into starts[0..m] (ghost export; one block)
__global__ void __launch_bounds__(1024) k_scan_plain(const int *count, int *start, int m) {
  __shared__ int warp_tot[32];
  __shared__ int carry_s;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  if (t == 0) carry_s = 0;
  __syncthreads();
  for (int base = 0; base < m; base += 1024) {
    const int k = base + t;
    const int s = k < m ? count[k] : 0;
    int inc = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(FULL_MASK, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane == 31) warp_tot[wid] = inc;
    __syncthreads();
    if (wid == 0) {
      int wv = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL_MASK, wv, o);
        if (lane >= o) wv += y;
      }
      warp_tot[lane] = wv;
    }
    __syncthreads();
    const int run = carry_s + inc - s + (wid ? warp_tot[wid - 1] : 0);
    if (k < m) start[k] = run;
    __syncthreads();
    if (t == 1023) carry_s = run + s;
    __syncthreads();
  }
  if (t == 0) start[m] = carry_s;
}

// ---------------------------------------------------------------------------
// upload of a single system (cavgpu_upload): host layouts to slot arrays on the device
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_upload_single(Dev d, Box b, int n, int ntypes, int has_vel, int has_id,
                                                       const double *raw_pos, const double *raw_vel,
                                                       const uint64_t *raw_type, const uint64_t *raw_id, int *seen,
                                                       int *type_count) {
  // per-type counts of the block in shared memory, one global atomic per type and
  // block (one per atom on a single address serialised the whole upload)
  __shared__ int s_count[CAVGPU_MAX_TYPES];
  if (threadIdx.x < CAVGPU_MAX_TYPES) s_count[threadIdx.x] = 0;
  __syncthreads();
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h < n) {
    const RepBox &rb = b.r0;
    const double x = raw_pos[3 * (size_t)h], y = raw_pos[3 * (size_t)h + 1], z = raw_pos[3 * (size_t)h + 2];
    // Atom_data::position_inside_global_domain (src/atom_data.cpp:548-559)
    bool bad = !(x >= rb.lo[0] && x < rb.hi[0] && y >= rb.lo[1] && y < rb.hi[1] && z >= rb.lo[2] && z < rb.hi[2]);
    const uint64_t t = raw_type[h];
    bad |= t >= (uint64_t)ntypes;
    const uint64_t id = has_id ? raw_id[h] : (uint64_t)h;
    if (id >= (uint64_t)n) bad = true;
    else if (atomicExch(&seen[id], 1) != 0) bad = true;  // ids: a permutation of 0..n-1
    if (bad) {
      d.flags[F_UPLOAD_BAD] = 1;
    } else {
      atomicAdd_block(&s_count[t], 1);
      d.pos[h] = make_dbl4(x, y, z, type_bits((int)t));
      d.vel[h] = has_vel ? make_dbl4(raw_vel[3 * (size_t)h], raw_vel[3 * (size_t)h + 1], raw_vel[3 * (size_t)h + 2],
                                     0.0)
                         : make_dbl4(0.0, 0.0, 0.0, 0.0);
      d.type[h] = (int)t;
      d.id[h] = (uint32_t)id;
    }
  }
  __syncthreads();
  if (threadIdx.x < CAVGPU_MAX_TYPES && s_count[threadIdx.x]) atomicAdd(&type_count[threadIdx.x], s_count[threadIdx.x]);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static inline int chk() { return cudaPeekAtLastError() == cudaSuccess ? CAVGPU_OK : CAVGPU_E_CUDA; }

int drift_grid_blocks(const LaunchCfg &lc) { return ceil_div(lc.n, 256); }

int launch_drift(const Dev &d, const Box &b, const StepConsts &sc, const LaunchCfg &lc, int k, int thermo,
                 cudaStream_t st) {
  const int g = drift_grid_blocks(lc);
  const bool mixed = lc.precision == CAVGPU_MIXED;
  if (lc.integrator == CAVGPU_VELOCITY_VERLET) {
    if (mixed) k_drift_vv<true><<<g, 256, 0, st>>>(d, b, sc);
    else k_drift_vv<false><<<g, 256, 0, st>>>(d, b, sc);
  } else if (lc.integrator == CAVGPU_LEAP_FROG) {
    if (mixed) k_drift_lf<true><<<g, 256, 0, st>>>(d, b, sc);
    else k_drift_lf<false><<<g, 256, 0, st>>>(d, b, sc);
  } else if (thermo < 0) {  // the velocity half only (constraint::Nve acts next)
    if (mixed) k_lang_a<true, false, false><<<g, 256, 0, st>>>(d, b, sc, k);
    else k_lang_a<false, false, false><<<g, 256, 0, st>>>(d, b, sc, k);
  } else {
    if (mixed) {
      if (thermo) k_lang_a<true, true, true><<<g, 256, 0, st>>>(d, b, sc, k);
      else k_lang_a<true, false, true><<<g, 256, 0, st>>>(d, b, sc, k);
    } else {
      if (thermo) k_lang_a<false, true, true><<<g, 256, 0, st>>>(d, b, sc, k);
      else k_lang_a<false, false, true><<<g, 256, 0, st>>>(d, b, sc, k);
    }
  }
  return chk();
}

int launch_lang_pos(const Dev &d, const Box &b, const StepConsts &sc, const LaunchCfg &lc, int thermo,
                    cudaStream_t st) {
  const int g = drift_grid_blocks(lc);
  if (lc.precision == CAVGPU_MIXED) {
    if (thermo) k_lang_pos<true, true><<<g, 256, 0, st>>>(d, b, sc);
    else k_lang_pos<true, false><<<g, 256, 0, st>>>(d, b, sc);
  } else {
    if (thermo) k_lang_pos<false, true><<<g, 256, 0, st>>>(d, b, sc);
    else k_lang_pos<false, false><<<g, 256, 0, st>>>(d, b, sc);
  }
  return chk();
}

int launch_rebuild(const Dev &d, const Box &b, const LaunchCfg &lc, int forced, cudaStream_t st) {
  const int g = ceil_div(b.nslot, 256);
  k_bin<<<g, 256, 0, st>>>(d, b, forced);
  const int P = scan_slices(b);
  if (P > 1) k_scan_part<<<P, 1024, 0, st>>>(d, b, forced);
  k_scan_rep<<<b.nrep * P, 1024, 0, st>>>(d, b, forced, P);
  k_scatter<<<g, 256, 0, st>>>(d, b, forced);
  k_cell_sort<<<ceil_div((long long)b.ncell_all * 32, 256), 256, 0, st>>>(d, b, forced);
  k_copy_state<<<g, 256, 0, st>>>(d, b, forced);
  k_gather<<<g, 256, 0, st>>>(d, b, forced);
  const int build_grid = std::min(ceil_div(ceil_div(b.nslot, 32), BUILD_WARPS), num_sms() * 8);
  if (lc.precision == CAVGPU_MIXED) k_build_group<1><<<build_grid, BUILD_WARPS * 32, 0, st>>>(d, b, forced);
  else k_build_group<0><<<build_grid, BUILD_WARPS * 32, 0, st>>>(d, b, forced);
  k_finish_rebuild<<<1, 256, 0, st>>>(d, b, forced);
  return chk();
}

int launch_set_rebuild_cond(const Dev &d, cudaGraphConditionalHandle h, cudaStream_t st) {
  k_set_rebuild_cond<<<1, 1, 0, st>>>(d, h);
  return chk();
}

int launch_halt_check(const Dev &d, cudaStream_t st) {
  k_halt_check<<<1, 1, 0, st>>>(d);
  return chk();
}

int launch_thermo_final(const Dev &d, const ThermoCfg &tc, int nb_ke, int nb_ev, int nb_ke_end, int ring_slot,
                        cudaStream_t st) {
  k_thermo_final<<<THERMO_FOLD_BLOCKS, 256, 0, st>>>(d, tc, nb_ke, nb_ev, nb_ke_end, ring_slot);
  return chk();
}

int launch_thermo_replicas(const Dev &d, const Box &b, const ThermoCfg &tc, int ke, int ev, cudaStream_t st) {
  k_thermo_rep<<<b.nrep, 256, 0, st>>>(d, b, tc, ke, ev);
  return chk();
}

int launch_advance_step(const Dev &d, cudaStream_t st) {
  k_advance_step<<<1, 1, 0, st>>>(d);
  return chk();
}

int launch_nve(const Dev &d, const Box &b, const ThermoCfg &tc, const NveCfg &cfg, int k, int thermo, int ring_slot,
               cudaStream_t st) {
  if (b.nrep != 1 || cfg.step <= 0) return CAVGPU_E_ARG;
  const int n = b.nslot;
  k_nve_ke<<<NVE_BLOCKS, 256, 0, st>>>(d, n, cfg, k);
  k_nve_lambda<<<1, 256, 0, st>>>(d, tc, cfg, k, thermo, ring_slot);
  k_nve_scale<<<NVE_BLOCKS, 256, 0, st>>>(d, n, cfg, k);
  return chk();
}

int launch_to_host_order(const Dev &d, const Box &b, int what, cudaStream_t st) {
  k_to_host_order<<<ceil_div(b.nslot, 256), 256, 0, st>>>(d, b, what);
  return chk();
}

int launch_images_to_host(const Dev &d, const Box &b, cudaStream_t st) {
  if (!d.img || !d.hi3) return CAVGPU_E_STATE;
  k_images_to_host<<<ceil_div(b.nslot, 256), 256, 0, st>>>(d, b);
  return chk();
}

int launch_export_pairs(const Dev &d, const Box &b, int mode, int32_t *rows, unsigned long long *counter,
                        int64_t cap, cudaStream_t st) {
  k_export_pairs<<<ceil_div(b.nslot, 256), 256, 0, st>>>(d, b, mode, rows, counter, (long long)cap);
  return chk();
}

int launch_ref_bins(const Dev &d, int n, double cutoff_inv, const int nb[3], const double lo_local[3],
                    cudaStream_t st) {
  RefBins rb;
  for (int a = 0; a < 3; ++a) { rb.lo[a] = lo_local[a]; rb.nb[a] = nb[a]; }
  rb.inv = cutoff_inv;
  k_ref_bins<<<ceil_div(n, 256), 256, 0, st>>>(d, n, rb);
  return chk();
}

int launch_upload_single(const Dev &d, const Box &b, int n, int ntypes, bool has_vel, bool has_id,
                         const double *raw_pos, const double *raw_vel, const uint64_t *raw_type,
                         const uint64_t *raw_id, int *seen, int *type_count, cudaStream_t st) {
  k_upload_single<<<ceil_div(n, 256), 256, 0, st>>>(d, b, n, ntypes, has_vel, has_id, raw_pos, raw_vel, raw_type,
                                                     raw_id, seen, type_count);
  return chk();
}

int launch_ghosts(const Dev &d, const Box &b, int n, double gc, int *counts, int *starts, int32_t *src,
                  int32_t *shift3, double *pos3, int32_t *bins3, int64_t cap, double cutoff_inv, const int nb[3],
                  const double lo_local[3], cudaStream_t st) {
  GhostCfg g;
  RefBins rb;
  for (int a = 0; a < 3; ++a) {
    g.llow[a] = b.r0.lo[a] + gc;
    g.lupp[a] = b.r0.hi[a] - gc;
    g.L[a] = b.r0.L[a];
    rb.lo[a] = lo_local[a];
    rb.nb[a] = nb[a];
  }
  rb.inv = cutoff_inv;
  k_ghost_count<<<ceil_div(n, 256), 256, 0, st>>>(d, n, g, counts);
  k_scan_plain<<<1, 1024, 0, st>>>(counts, starts, n);
  k_ghost_emit<<<ceil_div(n, 256), 256, 0, st>>>(d, n, g, starts, src, shift3, pos3, bins3, (long long)cap, rb);
  return chk();
}

}  // namespace cav
