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
  r.w = __int_as_float((int)x.w);
  d.rel[i] = r;
}

__device__ inline void request_rebuild(const Dev &d, const Box &b, int rep) {
  b.rep_flag[rep] = 1;
  d.flags[F_REBUILD] = 1;
}

__device__ inline void half_skin_test(const Dev &d, const Box &b, int rep, int i, const dbl4 &x) {
  const dbl4 r = d.pos_ref[i];
  const double dx = x.x - r.x, dy = x.y - r.y, dz = x.z - r.z;
  if (dx * dx + dy * dy + dz * dz > b.thr2) request_rebuild(d, b, rep);
}

// Mixed form: the displacement since the build is taken once in FP64 (3
// subtractions) and serves both the half-skin test (in FP32 against a threshold
// shrunk by 1e-6, so it can only fire early) and the FP32 cell-relative
// coordinates, rel = rel_at_build + (float)(x - x_at_build).
__device__ inline void mixed_track(const Dev &d, const Box &b, int rep, int i, const dbl4 &x) {
  const dbl4 r = d.pos_ref[i];
  const float fx = (float)(x.x - r.x), fy = (float)(x.y - r.y), fz = (float)(x.z - r.z);
  if (fx * fx + fy * fy + fz * fz > b.thr2f) request_rebuild(d, b, rep);
  const float4 q = d.rel_ref[i];
  d.rel[i] = make_float4(q.x + fx, q.y + fy, q.z + fz, q.w);
}

__device__ inline void nan_check(const Dev &d, int i, const dbl4 &a) {
  if (isnan(a.x) || isnan(a.y) || isnan(a.z)) {
    d.flags[F_NAN] = 1;
    d.flags[F_NAN_ATOM] = (int)d.id[i];
  }
}

// FP64 form: pos += vel*dt + ((acc*0.5)*dt)*dt, unfused, in the reference's order
// (src/md_simulator.cpp:654), so that equal forces give equal trajectories.
// Mixed form: the same update with two FMAs per component (the FP64 pipe of
// this part is its scarcest resource).
template <bool MIXED>
__global__ void __launch_bounds__(256) k_drift_vv(Dev d, Box b, StepConsts sc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= sc.n) return;
  const int rep = rep_of_slot(b, i);
  if (rep < 0) return;  // padding slot
  dbl4 x = d.pos[i];
  const dbl4 v = d.vel[i], a = d.acc[i];
  nan_check(d, i, a);
  if (MIXED) {
    x.x = fma(a.x, sc.hdt2, fma(v.x, sc.dt, x.x));
    x.y = fma(a.y, sc.hdt2, fma(v.y, sc.dt, x.y));
    x.z = fma(a.z, sc.hdt2, fma(v.z, sc.dt, x.z));
  } else {
    x.x = __dadd_rn(x.x, __dadd_rn(__dmul_rn(v.x, sc.dt), __dmul_rn(__dmul_rn(__dmul_rn(a.x, 0.5), sc.dt), sc.dt)));
    x.y = __dadd_rn(x.y, __dadd_rn(__dmul_rn(v.y, sc.dt), __dmul_rn(__dmul_rn(__dmul_rn(a.y, 0.5), sc.dt), sc.dt)));
    x.z = __dadd_rn(x.z, __dadd_rn(__dmul_rn(v.z, sc.dt), __dmul_rn(__dmul_rn(__dmul_rn(a.z, 0.5), sc.dt), sc.dt)));
  }
  d.pos[i] = x;  // acc stays: the pair kernel's kick reads it as a_old
  if (MIXED) mixed_track(d, b, rep, i, x);
  else half_skin_test(d, b, rep, i, x);
}

// Leap-frog first half (src/md_simulator.cpp:890-905): v += (0.5 dt) a ; r += dt v.
// The closing half, v += (0.5 dt) a(t + dt), is the velocity-Verlet kick of the pair
// kernel with a_old = 0: v + (a + 0)(0.5 dt) rounds exactly as v + (0.5 dt) a.
template <bool MIXED>
__global__ void __launch_bounds__(256) k_drift_lf(Dev d, Box b, StepConsts sc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= sc.n) return;
  const int rep = rep_of_slot(b, i);
  if (rep < 0) return;  // padding slot
  dbl4 x = d.pos[i], v = d.vel[i];
  const dbl4 a = d.acc[i];
  nan_check(d, i, a);
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
  d.pos[i] = x;
  d.vel[i] = v;
  d.acc[i] = make_dbl4(0.0, 0.0, 0.0, 0.0);  // a_old = 0 for the kick
  if (MIXED) mixed_track(d, b, rep, i, x);
  else half_skin_test(d, b, rep, i, x);
}

// Langevin position update r += v*c (src/md_simulator.cpp:822-827) with the
// half-skin tracking; with THERMO the temperature sums of the velocities first.
template <bool MIXED, bool THERMO>
__device__ __forceinline__ void lang_position(const Dev &d, const Box &b, const StepConsts &sc, int rep, int i, dbl4 x,
                                              const dbl4 &v, double (&part)[4]) {
  if (THERMO) {
    const double m = d.tab->mass[(int)x.w];
    part[0] = m * (v.x * v.x + v.y * v.y + v.z * v.z);
    part[1] = m * v.x; part[2] = m * v.y; part[3] = m * v.z;
  }
  if (MIXED) {
    x.x = fma(v.x, sc.lc, x.x);
    x.y = fma(v.y, sc.lc, x.y);
    x.z = fma(v.z, sc.lc, x.z);
  } else {
    x.x = __dadd_rn(x.x, __dmul_rn(v.x, sc.lc));
    x.y = __dadd_rn(x.y, __dmul_rn(v.y, sc.lc));
    x.z = __dadd_rn(x.z, __dmul_rn(v.z, sc.lc));
  }
  d.pos[i] = x;
  if (MIXED) mixed_track(d, b, rep, i, x);
  else half_skin_test(d, b, rep, i, x);
}

// Langevin first half (src/md_simulator.cpp:748-837):
//   v += (a*0.5)*dt + eta*b ; [temperature here] ; r += v*c
// POS false: the velocity half only; constraint::Nve then acts on the mid-step
// velocities (:784-791) and k_lang_pos takes the temperature and moves the atoms.
template <bool MIXED, bool THERMO, bool POS>
__global__ void __launch_bounds__(256) k_lang_a(Dev d, Box b, StepConsts sc, int k_in_chunk) {
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
    if (MIXED) {
      v.x = fma(a.x, sc.hdt, fma(e0, sc.lb, v.x));
      v.y = fma(a.y, sc.hdt, fma(e1, sc.lb, v.y));
      v.z = fma(a.z, sc.hdt, fma(e2, sc.lb, v.z));
    } else {
      v.x = __dadd_rn(v.x, __dadd_rn(__dmul_rn(__dmul_rn(a.x, 0.5), sc.dt), __dmul_rn(e0, sc.lb)));
      v.y = __dadd_rn(v.y, __dadd_rn(__dmul_rn(__dmul_rn(a.y, 0.5), sc.dt), __dmul_rn(e1, sc.lb)));
      v.z = __dadd_rn(v.z, __dadd_rn(__dmul_rn(__dmul_rn(a.z, 0.5), sc.dt), __dmul_rn(e2, sc.lb)));
    }
    d.vel[i] = v;
    if (POS) lang_position<MIXED, THERMO>(d, b, sc, rep, i, x, v, part);
  }
  if (POS && THERMO) block_sum_store<4>(part, &d.partials_ke[(size_t)blockIdx.x * 4]);
}

template <bool MIXED, bool THERMO>
__global__ void __launch_bounds__(256) k_lang_pos(Dev d, Box b, StepConsts sc) {
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
__device__ inline bool rebuild_on(const Box &b, int rep, int forced) { return forced || b.rep_flag[rep] != 0; }

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
  const bool act = rep >= 0 && rebuild_on(b, rep, forced);
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
  if (!rebuild_on(b, 0, forced)) return;
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
  if (!rebuild_on(b, rep, forced)) return;
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
  if (rep < 0 || !rebuild_on(b, rep, forced)) return;
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
  if (rep < 0 || !rebuild_on(b, rep, forced)) return;
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
  if (rep < 0 || !rebuild_on(b, rep, forced)) return;
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
  if (rep < 0 || !rebuild_on(b, rep, forced)) return;
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

// Stencil cell k of home cell (cx, cy, cz): its global index, its periodic image
// code and the offset of its origin from the home cell's origin.
struct StencilCell {
  int c2, img;
  float ox, oy, oz;
};
__device__ inline StencilCell stencil_cell(const RepBox &rb, int cx, int cy, int cz, int k) {
  const int dx = k % 3 - 1, dy = (k / 3) % 3 - 1, dz = k / 9 - 1;
  int nx = cx + dx, ny = cy + dy, nz = cz + dz, sx = 0, sy = 0, sz = 0;
  if (nx < 0) { nx += rb.nc[0]; sx = -1; } else if (nx >= rb.nc[0]) { nx -= rb.nc[0]; sx = 1; }
  if (ny < 0) { ny += rb.nc[1]; sy = -1; } else if (ny >= rb.nc[1]) { ny -= rb.nc[1]; sy = 1; }
  if (nz < 0) { nz += rb.nc[2]; sz = -1; } else if (nz >= rb.nc[2]) { nz -= rb.nc[2]; sz = 1; }
  StencilCell s;
  s.c2 = rb.cell_off + nx + rb.nc[0] * (ny + rb.nc[1] * nz);
  s.img = image_code(sx, sy, sz);
  s.ox = dx * rb.wf[0];
  s.oy = dy * rb.wf[1];
  s.oz = dz * rb.wf[2];
  return s;
}

// One warp per home cell, one lane per home atom (cells of more than 32 atoms
// take several groups).  The warp first stages the 27 stencil cells' atoms, in
// stencil order and slot order inside a cell, into its slice of shared memory,
// candidates u and u+1 (u even) interleaved as {x_u, x_u+1, y_u, y_u+1} and
// {z_u, z_u+1, word_u, word_u+1} (coordinates relative to the home cell's origin,
// word = j | code), padded to a multiple of 32 with far-away entries; stencils of
// more than BUILD_STAGE candidates are staged in passes.  The sweep takes 32
// candidates at a time, two per packed FP32x2 distance evaluation: every pair of
// candidates is two shared-memory broadcasts tested by all home atoms, the results
// collect in a hit and a band bit mask per lane (one warp vote per 32 candidates
// for the rare exact FP64 test), and only then are the hits (~15% of the
// candidates) written, in candidate order.  Hits append to the lane's own row, so
// the list keeps the stencil order (deterministic, independent of the launch shape).
constexpr int BUILD_WARPS = 8;    // warps per block
constexpr int BUILD_STAGE = 256;  // staged candidates per warp and pass (4 KiB)

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

__global__ void __launch_bounds__(BUILD_WARPS * 32, 4) k_build_warp(Dev d, Box b, int mode, int forced) {
  __shared__ float4 stage_all[BUILD_WARPS][BUILD_STAGE];
  const int lane = threadIdx.x & 31;
  // pair p = candidates 2p, 2p+1: sxy[p] = {x, x', y, y'}, szw[p] = {z, z', word, word'}
  float4 *sxy = stage_all[threadIdx.x >> 5], *szw = sxy + BUILD_STAGE / 2;
  float *fxy = reinterpret_cast<float *>(sxy), *fzw = reinterpret_cast<float *>(szw);
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  const int cap = d.cap;
  const int cshift = 7 - log2_pow2(d.tpa);  // chunk stride 4A words = 2^(log2 A + 2)
  int wmax = 0;
  for (int cell = gw; cell < b.ncell_all; cell += nw) {
    const int rep = rep_of_cell(b, cell);
    if (rep < 0 || !rebuild_on(b, rep, forced)) continue;
    const RepBox &rb = repbox(b, rep);
    const int lc = cell - rb.cell_off;
    if (lc >= rb.ncell) continue;  // the padding cell
    const int hs = d.cell_start[cell], he = d.cell_start[cell + 1];
    const int cx = lc % rb.nc[0], cy = (lc / rb.nc[0]) % rb.nc[1], cz = lc / (rb.nc[0] * rb.nc[1]);
    // lane k < 27: stencil cell k's first slot and count (exclusive scan = its
    // position in the flattened candidate sequence), list-word code and origin offset
    int kb = 0, kn = 0;
    uint32_t kcode = 0u;
    float kox = 0.f, koy = 0.f, koz = 0.f;
    if (lane < 27) {
      const StencilCell s = stencil_cell(rb, cx, cy, cz, lane);
      kb = d.cell_start[s.c2];
      kn = d.cell_start[s.c2 + 1] - kb;
      kcode = (uint32_t)(mode == 0 ? s.img : lane) << CODE_SHIFT;
      kox = s.ox; koy = s.oy; koz = s.oz;
    }
    int kpre = kn;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(FULL_MASK, kpre, o);
      if (lane >= o) kpre += y;
    }
    const int ntot = __shfl_sync(FULL_MASK, kpre, 26);
    kpre -= kn;
    const int k13 = __shfl_sync(FULL_MASK, kpre, 13);  // where the home cell's atoms start
    for (int h0 = hs; h0 < he; h0 += 32) {
      const int i = h0 + lane;
      const bool act = i < he;
      const float4 ri = act ? d.rel[i] : make_float4(0.f, 0.f, 0.f, 0.f);
      const unsigned long long rxx = pack2(ri.x), ryy = pack2(ri.y), rzz = pack2(ri.z);
      const float lo = b.ce2_lo;
      const float hi = act ? b.ce2_hi : -1.0f;  // idle lanes never hit
      // the atom itself: stencil cell 13 (the home cell, image zero), at its rank in the cell
      const int tself = act ? k13 + (i - hs) : -1;
      const int mol_i = d.mol && act ? d.mol[i] : 0;
      uint32_t *row = d.nbr + nbr_block_base(act ? i : hs, cap, d.tpa);
      int cnt = 0;
      for (int p0 = 0; p0 < ntot; p0 += BUILD_STAGE) {
        const int np = min(BUILD_STAGE, ntot - p0);
        __syncwarp();
        for (int k = 0; k < 27; ++k) {
          const int f0 = __shfl_sync(FULL_MASK, kpre, k), cn = __shfl_sync(FULL_MASK, kn, k);
          const int lo_t = max(f0, p0), hi_t = min(f0 + cn, p0 + np);
          if (lo_t >= hi_t) continue;
          const int jb = __shfl_sync(FULL_MASK, kb, k);
          const uint32_t code = __shfl_sync(FULL_MASK, kcode, k);
          const float ox = __shfl_sync(FULL_MASK, kox, k), oy = __shfl_sync(FULL_MASK, koy, k),
                      oz = __shfl_sync(FULL_MASK, koz, k);
          for (int t = lo_t + lane; t < hi_t; t += 32) {
            const int j = jb + (t - f0);
            const float4 rj = __ldg(&d.rel[j]);
            const int e = ((t - p0) >> 1) * 4 + ((t - p0) & 1);
            fxy[e] = rj.x + ox;
            fxy[e + 2] = rj.y + oy;
            fzw[e] = rj.z + oz;
            fzw[e + 2] = __uint_as_float((uint32_t)j | code);
          }
        }
        const int npad32 = (np + 31) & ~31;
        for (int t = np + lane; t < npad32; t += 32) {
          const int e = (t >> 1) * 4 + (t & 1);
          fxy[e] = 1e18f;
          fxy[e + 2] = 1e18f;
          fzw[e] = 1e18f;
          fzw[e + 2] = 0.f;
        }
        __syncwarp();
        for (int t0 = 0; t0 < npad32; t0 += 32) {
          // phase 1: bits of the sure hits (q < ce2_lo) and of everything up to ce2_hi
          uint32_t hm = 0u, am = 0u;
#pragma unroll
          for (int u = 0; u < 32; u += 2) {
            const int pr = (t0 + u) >> 1;
            const float4 xy = sxy[pr];                                  // broadcast
            const float2 z = *reinterpret_cast<const float2 *>(&szw[pr]);  // broadcast
            float q0, q1;
            dist2_pair(xy, z, rxx, ryy, rzz, q0, q1);
            if (q0 < lo) hm |= 1u << u;
            if (q0 <= hi) am |= 1u << u;
            if (q1 < lo) hm |= 2u << u;
            if (q1 <= hi) am |= 2u << u;
          }
          const int ts = tself - (p0 + t0);  // the atom itself is no candidate
          if (ts >= 0 && ts < 32) am &= ~(1u << ts);
          hm &= am;
          uint32_t bm = am & ~hm;  // the band
          if (__any_sync(FULL_MASK, bm != 0u)) {  // rare: the exact FP64 predicate
            while (bm) {
              const int u = __ffs(bm) - 1;
              bm &= bm - 1u;
              const uint32_t w = __float_as_uint(fzw[((t0 + u) >> 1) * 4 + 2 + (u & 1)]);
              const int code = (int)(w >> CODE_SHIFT);
              int img = code;
              if (mode != 0) {  // recover the image from the stencil index
                const int nx = cx + code % 3 - 1, ny = cy + (code / 3) % 3 - 1, nz = cz + code / 9 - 1;
                img = image_code(nx < 0 ? -1 : (nx >= rb.nc[0] ? 1 : 0), ny < 0 ? -1 : (ny >= rb.nc[1] ? 1 : 0),
                                 nz < 0 ? -1 : (nz >= rb.nc[2] ? 1 : 0));
              }
              if (exact_pair(d, rb, b.ce2, i, (int)(w & IDX_MASK), img)) hm |= 1u << u;
            }
          }
          // phase 2: the hits, in candidate order (ignore_intra_molecule: none of the
          // atom's own molecule, as Lj::calculate_acceleration skips them, lj.cpp:446)
          while (hm) {
            const int u = __ffs(hm) - 1;
            hm &= hm - 1u;
            const uint32_t w = __float_as_uint(fzw[((t0 + u) >> 1) * 4 + 2 + (u & 1)]);
            if (d.mol && d.mol[w & IDX_MASK] == mol_i) continue;
            if (cnt < cap) row[((cnt >> 2) << cshift) + (cnt & 3)] = w;
            ++cnt;
          }
        }
      }
      if (act) {
        d.nnbr[i] = min(cnt, cap);
        if (cnt > cap) atomicMax(&d.flags[F_OVERFLOW], cnt);
        wmax = max(wmax, cnt);
      }
    }
  }
  // one atomic per warp for the largest list length (not one per atom)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(FULL_MASK, wmax, o));
  if (lane == 0 && wmax > 0) atomicMax(&d.flags[F_MAXNB], wmax);
}

// after the build: count the rebuilt replicas, clear their flags and the global one
__global__ void __launch_bounds__(256) k_finish_rebuild(Dev d, Box b, int forced) {
  __shared__ int total;
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  int n = 0;
  for (int r = threadIdx.x; r < b.nrep; r += blockDim.x) {
    n += rebuild_on(b, r, forced) ? 1 : 0;
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
  }
}

// Inside a captured step: the half-skin flag becomes the value of the graph's
// conditional node that wraps the rebuild kernels.
__global__ void k_set_rebuild_cond(Dev d, cudaGraphConditionalHandle h) {
  cudaGraphSetConditional(h, d.flags[F_REBUILD] != 0 ? 1u : 0u);
}

// ---------------------------------------------------------------------------
// thermo: fold the per-block partials (fixed order) into KE, T, P, virial, PE
// (Atom_data::kinetic_energy_mpi_domain / finalize_temperature / finalize_pressure,
//  src/atom_data/kinetic_energy.cpp:26-134, 189-198, 238-303)
// thermo[] = {KE, T, P, virial, PE, sum m, -, -}
// ---------------------------------------------------------------------------
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

__global__ void __launch_bounds__(256) k_thermo_final(Dev d, ThermoCfg tc, int nb_ke, int nb_ev, int nb_ke_end,
                                                      int ring_slot) {
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
  // level 2, in the last block: the blocks' sums in block order
  if (threadIdx.x < 10) {
    __threadfence();
    const volatile double *f = d.fold;
    double s = 0.0;
    for (int g = 0; g < (int)gridDim.x; ++g) s += f[g * 10 + threadIdx.x];
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

__global__ void k_advance_step(Dev d, int nsteps) { *d.step_base += nsteps; }

// ---------------------------------------------------------------------------
// constraint::Nve (src/constraint/nve.cpp:132-184), single system: on steps whose
// index is a multiple of `step`, lambda = sqrt(target / KE) with KE the kinetic
// energy of Atom_data::kinetic_energy (centre-of-mass part removed for n_r_df
// 1..3), velocities scaled by lambda, then the temperature and pressure of the
// step follow the scaled velocities (finalize_temperature / finalize_pressure).
// ---------------------------------------------------------------------------
__device__ inline bool nve_applies(const Dev &d, const NveCfg &c, int k) { return (*d.step_base + k) % c.step == 0; }

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
  const int mode = lc.precision == CAVGPU_MIXED ? 1 : 0;
  const int build_grid = std::min(ceil_div(b.ncell_all, BUILD_WARPS), num_sms() * 8);
  k_build_warp<<<build_grid, BUILD_WARPS * 32, 0, st>>>(d, b, mode, forced);
  k_finish_rebuild<<<1, 256, 0, st>>>(d, b, forced);
  return chk();
}

int launch_set_rebuild_cond(const Dev &d, cudaGraphConditionalHandle h, cudaStream_t st) {
  k_set_rebuild_cond<<<1, 1, 0, st>>>(d, h);
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

int launch_advance_step(const Dev &d, int nsteps, cudaStream_t st) {
  k_advance_step<<<1, 1, 0, st>>>(d, nsteps);
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
