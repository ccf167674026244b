// cav_force.cu -- the shifted-force LJ pair kernels (force_field::Lj::calculate_acceleration,
// src/force/lj.cpp:393-517), fused with the closing integrator update of the step.
//
// Full neighbour list, gather only (no atomics, deterministic): TPA lanes work on one
// atom, a warp on A = 32/TPA atoms, and the list layout (nbr_index) makes every
// iteration one coalesced 128-byte read of neighbour words.  Two precisions:
//   FP64  : image = x_j + s*L, all pair arithmetic in double;
//   MIXED : FP32 pair arithmetic on coordinates relative to each atom's build cell
//           (float4 x,y,z,type; cell offsets from a shared table), FP64 accumulation
//           across lanes, FP64 acceleration/velocity/reductions.
#include "cav_common.cuh"

namespace cav {

#define FULL_MASK 0xffffffffu

template <int NV>
__device__ inline void block_sum_store_f(double (&v)[NV], double *out) {
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
  if (threadIdx.x == 0)
    for (int k = 0; k < NV; ++k) {
      double s = 0.0;
      for (int w = 0; w < nw; ++w) s += sh[w][k];
      out[k] = s;
    }
}

struct SmemTabD {
  double rc2[MAXT * MAXT], sig2[MAXT * MAXT], eps4[MAXT * MAXT], gc[MAXT * MAXT], uc[MAXT * MAXT];
  double minv[MAXT], mass[MAXT];
};
struct SmemTabF {
  float rc2[MAXT * MAXT], sig2[MAXT * MAXT], eps4[MAXT * MAXT], gc[MAXT * MAXT], uc[MAXT * MAXT];
  double minv[MAXT], mass[MAXT];
};
// per warp: the 27 image shifts s*L (FP64) or cell offsets d*w (mixed) of the
// replica the warp's current atoms belong to (a warp never straddles two).  The
// mixed offsets are FP32 pairs d*wf + d*wlo: with the rounded width alone, every
// pair across a cell face would be displaced by the same d*(wf - w), a fixed
// distortion of the potential that changes pattern at each rebuild and drifts
// the NVE energy (measured -2.4e-4 per 1e6 steps).
template <bool MIXED>
struct WarpImages;
template <>
struct WarpImages<true> {
  float3 v[27];
  float3 lo[27];
};
template <>
struct WarpImages<false> {
  double3 v[27];
};

// KICK: 0 = store the acceleration only; 1 = velocity-Verlet closing kick
// v += (a + a_old) * (0.5 dt) (src/md_simulator.cpp:672-679); 2 = Langevin closing
// update v = (v a_L + eta b) + (a*0.5) dt (src/md_simulator.cpp:853-862).
// EV: accumulate virial and potential energy (and KE unless KICK == 2); batches
// also store them per slot for the per-replica folds.
template <int TPA, bool MIXED, int KICK, bool EV>
__global__ void __launch_bounds__(256) k_force(Dev d, Box b, StepConsts sc, int k_in_chunk) {
  constexpr int A = 32 / TPA;
  __shared__ typename std::conditional<MIXED, SmemTabF, SmemTabD>::type tab;
  __shared__ WarpImages<MIXED> wimg[8];
  const PairTab &T = *d.tab;
  const int nt = T.nt;
  for (int k = threadIdx.x; k < nt * nt; k += blockDim.x) {
    tab.rc2[k] = T.rc2[k]; tab.sig2[k] = T.sig2[k]; tab.eps4[k] = T.eps4[k]; tab.gc[k] = T.gc[k];
    tab.uc[k] = T.uc[k];
  }
  for (int k = threadIdx.x; k < nt; k += blockDim.x) { tab.minv[k] = T.minv[k]; tab.mass[k] = T.mass[k]; }
  __syncthreads();

  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int a = lane % A, t = lane / A;
  const int n = sc.n, cap = d.cap;
  const int warps_total = (gridDim.x * blockDim.x) >> 5;
  const int ntask = (n + A - 1) / A;
  double ke_p[4] = {0.0, 0.0, 0.0, 0.0};
  double ev_p[2] = {0.0, 0.0};
  long long step = 0;
  if (KICK == 2) step = *d.step_base + k_in_chunk;
  auto &img = wimg[wid].v;
  int img_rep = -1;

  for (int task = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; task < ntask; task += warps_total) {
    const int rep = rep_of_slot(b, task * A);
    if (rep < 0) continue;  // a task of padding slots (uniform over the warp)
    if (rep != img_rep) {
      const RepBox &rb = repbox(b, rep);
      if (lane < 27) {
        const int sx = lane % 3 - 1, sy = (lane / 3) % 3 - 1, sz = lane / 9 - 1;
        if constexpr (MIXED) {
          img[lane] = make_float3(sx * rb.wf[0], sy * rb.wf[1], sz * rb.wf[2]);
          wimg[wid].lo[lane] = make_float3(sx * rb.wlo[0], sy * rb.wlo[1], sz * rb.wlo[2]);
        } else {
          img[lane] = make_double3(sx * rb.L[0], sy * rb.L[1], sz * rb.L[2]);
        }
      }
      __syncwarp();
      img_rep = rep;
    }
    const int i = task * A + a;
    const bool act = i < n && rep_of_slot(b, i) >= 0;
    double fx = 0.0, fy = 0.0, fz = 0.0, vir = 0.0, pe = 0.0;
    int ti = 0;
    if (act) {
      const int nn = d.nnbr[i];
      // this lane's neighbour words: chunk g = t + TPA q (entries 4g..4g+3), one 128-bit
      // load each; the warp's loads for one q cover 512 consecutive bytes (nbr_index)
      const uint4 *row4 = reinterpret_cast<const uint4 *>(d.nbr + (size_t)task * cap * A) + (t * A + a);
      if constexpr (MIXED) {
        const float4 ri = d.rel[i];
        ti = __float_as_int(ri.w);
        float ax = 0.f, ay = 0.f, az = 0.f, vr = 0.f, pp = 0.f;
        for (int q = 0, k0 = 4 * t; k0 < nn; ++q, k0 += 4 * TPA) {
          const uint4 w4 = __ldg(row4 + (size_t)q * 32);
          const uint32_t e[4] = {w4.x, w4.y, w4.z, w4.w};
          float4 rj[4];
#pragma unroll
          for (int u = 0; u < 4; ++u)  // four independent gathers in flight
            if (k0 + u < nn) rj[u] = __ldg(&d.rel[e[u] & IDX_MASK]);
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            if (k0 + u >= nn) break;
            // ((r_j - r_i) + offset_hi) + offset_lo: rounding is symmetric under negation
            // and the offsets of i seen from j are exactly -offset, so d_ji = -d_ij bit
            // for bit and the FP32 pair forces obey Newton's third law exactly
            const int code = e[u] >> CODE_SHIFT;
            const float3 o = img[code], ol = wimg[wid].lo[code];
            const float dx = ((rj[u].x - ri.x) + o.x) + ol.x, dy = ((rj[u].y - ri.y) + o.y) + ol.y,
                        dz = ((rj[u].z - ri.z) + o.z) + ol.z;
            const float r2 = dx * dx + dy * dy + dz * dz;
            const int tt = ti * nt + __float_as_int(rj[u].w);
            if (r2 <= tab.rc2[tt]) {
              const float r2i = __frcp_rn(r2);
              const float s2 = tab.sig2[tt] * r2i;
              const float s6 = s2 * s2 * s2;
              const float coef = tab.eps4[tt] * r2i * s6 * (6.0f - 12.0f * s6) - tab.gc[tt];
              ax += coef * dx; ay += coef * dy; az += coef * dz;
              if (EV) {
                vr -= coef * r2;
                pp += tab.eps4[tt] * (s6 * s6 - s6) - tab.uc[tt] - 0.5f * tab.gc[tt] * (r2 - tab.rc2[tt]);
              }
            }
          }
        }
        fx = ax; fy = ay; fz = az; vir = vr; pe = pp;
      } else {
        const dbl4 xi = d.pos[i];
        ti = (int)xi.w;
        for (int q = 0, k0 = 4 * t; k0 < nn; ++q, k0 += 4 * TPA) {
          const uint4 w4 = __ldg(row4 + (size_t)q * 32);
          const uint32_t e[4] = {w4.x, w4.y, w4.z, w4.w};
          dbl4 xj[4];
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (k0 + u < nn) xj[u] = ldg_dbl4(&d.pos[e[u] & IDX_MASK]);
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            if (k0 + u >= nn) break;
            const double3 s = img[e[u] >> CODE_SHIFT];
            const double dx = (xj[u].x + s.x) - xi.x, dy = (xj[u].y + s.y) - xi.y, dz = (xj[u].z + s.z) - xi.z;
            const double r2 = dx * dx + dy * dy + dz * dz;
            const int tt = ti * nt + (int)xj[u].w;
            if (r2 <= tab.rc2[tt]) {
              const double r2i = __drcp_rn(r2);
              const double s2 = tab.sig2[tt] * r2i;
              const double s6 = s2 * s2 * s2;
              const double coef = tab.eps4[tt] * r2i * s6 * (6.0 - 12.0 * s6) - tab.gc[tt];
              fx += coef * dx; fy += coef * dy; fz += coef * dz;
              if (EV) {
                vir -= coef * r2;
                pe += tab.eps4[tt] * (s6 * s6 - s6) - tab.uc[tt] - 0.5 * tab.gc[tt] * (r2 - tab.rc2[tt]);
              }
            }
          }
        }
      }
    }
    // fold the TPA lanes of each atom (lanes a, a+A, a+2A, ...)
#pragma unroll
    for (int o = A; o < 32; o <<= 1) {
      fx += __shfl_xor_sync(FULL_MASK, fx, o);
      fy += __shfl_xor_sync(FULL_MASK, fy, o);
      fz += __shfl_xor_sync(FULL_MASK, fz, o);
      if (EV) {
        vir += __shfl_xor_sync(FULL_MASK, vir, o);
        pe += __shfl_xor_sync(FULL_MASK, pe, o);
      }
    }
    if (act && t == 0) {
      const double mi = tab.minv[ti];
      dbl4 an = make_dbl4(fx * mi, fy * mi, fz * mi, 0.0);
      if (KICK == 0) {
        d.acc[i] = an;
        if (EV) {
          const dbl4 v = d.vel[i];
          const double m = tab.mass[ti];
          ke_p[0] += m * (v.x * v.x + v.y * v.y + v.z * v.z);
          ke_p[1] += m * v.x; ke_p[2] += m * v.y; ke_p[3] += m * v.z;
        }
      } else if (KICK == 1) {
        dbl4 v = d.vel[i];
        const dbl4 ao = d.acc_old[i];
        if (MIXED) {
          v.x = fma(an.x + ao.x, sc.hdt, v.x);
          v.y = fma(an.y + ao.y, sc.hdt, v.y);
          v.z = fma(an.z + ao.z, sc.hdt, v.z);
        } else {  // v += (a + a_old) * (0.5 dt), the reference's order
          v.x = __dadd_rn(v.x, __dmul_rn(__dadd_rn(an.x, ao.x), sc.hdt));
          v.y = __dadd_rn(v.y, __dmul_rn(__dadd_rn(an.y, ao.y), sc.hdt));
          v.z = __dadd_rn(v.z, __dmul_rn(__dadd_rn(an.z, ao.z), sc.hdt));
        }
        d.acc[i] = an;
        d.vel[i] = v;
        if (EV) {
          const double m = tab.mass[ti];
          ke_p[0] += m * (v.x * v.x + v.y * v.y + v.z * v.z);
          ke_p[1] += m * v.x; ke_p[2] += m * v.y; ke_p[3] += m * v.z;
        }
      } else {
        dbl4 v = d.vel[i];
        double e0 = 0.0, e1 = 0.0, e2 = 0.0;
        if (!sc.noise_off) {
          if (MIXED) langevin_eta_f(sc.seed + rep, step, d.id[i], e0, e1, e2);
          else langevin_eta(sc.seed + rep, step, d.id[i], e0, e1, e2);
        }
        if (MIXED) {
          v.x = fma(an.x, sc.hdt, fma(v.x, sc.la, e0 * sc.lb));
          v.y = fma(an.y, sc.hdt, fma(v.y, sc.la, e1 * sc.lb));
          v.z = fma(an.z, sc.hdt, fma(v.z, sc.la, e2 * sc.lb));
        } else {  // v = (v a + eta b) + (a*0.5) dt, the reference's order
          v.x = __dadd_rn(__dadd_rn(__dmul_rn(v.x, sc.la), __dmul_rn(e0, sc.lb)), __dmul_rn(__dmul_rn(an.x, 0.5), sc.dt));
          v.y = __dadd_rn(__dadd_rn(__dmul_rn(v.y, sc.la), __dmul_rn(e1, sc.lb)), __dmul_rn(__dmul_rn(an.y, 0.5), sc.dt));
          v.z = __dadd_rn(__dadd_rn(__dmul_rn(v.z, sc.la), __dmul_rn(e2, sc.lb)), __dmul_rn(__dmul_rn(an.z, 0.5), sc.dt));
        }
        d.acc[i] = an;
        d.vel[i] = v;
      }
      if (EV) {
        ev_p[0] += vir;
        ev_p[1] += pe;
        if (d.ev_atom) d.ev_atom[i] = make_double2(vir, pe);
      }
    }
  }
  if (EV) {
    block_sum_store_f<2>(ev_p, &d.partials_ev[(size_t)blockIdx.x * 2]);
    if (KICK != 2) {
      __syncthreads();
      block_sum_store_f<4>(ke_p, &d.partials_ke[(size_t)blockIdx.x * 4]);
    }
  }
}

template <int TPA, bool MIXED, int KICK>
static void launch_ev(bool ev, int grid, int block, const Dev &d, const Box &b, const StepConsts &sc, int k,
                      cudaStream_t st) {
  if (ev) k_force<TPA, MIXED, KICK, true><<<grid, block, 0, st>>>(d, b, sc, k);
  else k_force<TPA, MIXED, KICK, false><<<grid, block, 0, st>>>(d, b, sc, k);
}

template <int TPA, bool MIXED>
static void launch_kick(int kick, bool ev, int grid, int block, const Dev &d, const Box &b, const StepConsts &sc,
                        int k, cudaStream_t st) {
  if (kick == 0) launch_ev<TPA, MIXED, 0>(ev, grid, block, d, b, sc, k, st);
  else if (kick == 1) launch_ev<TPA, MIXED, 1>(ev, grid, block, d, b, sc, k, st);
  else launch_ev<TPA, MIXED, 2>(ev, grid, block, d, b, sc, k, st);
}

template <bool MIXED>
static int launch_tpa(int tpa, int kick, bool ev, int grid, int block, const Dev &d, const Box &b,
                      const StepConsts &sc, int k, cudaStream_t st) {
  switch (tpa) {
    case 1: launch_kick<1, MIXED>(kick, ev, grid, block, d, b, sc, k, st); break;
    case 2: launch_kick<2, MIXED>(kick, ev, grid, block, d, b, sc, k, st); break;
    case 4: launch_kick<4, MIXED>(kick, ev, grid, block, d, b, sc, k, st); break;
    case 8: launch_kick<8, MIXED>(kick, ev, grid, block, d, b, sc, k, st); break;
    case 16: launch_kick<16, MIXED>(kick, ev, grid, block, d, b, sc, k, st); break;
    default: return CAVGPU_E_ARG;
  }
  return CAVGPU_OK;
}

static int g_num_sms = 0;

int force_grid_blocks(const LaunchCfg &lc) {
  if (!g_num_sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 148;
  }
  const int A = 32 / lc.tpa;
  const long long ntask = (lc.n + A - 1) / A;
  const long long warps_per_block = lc.block / 32;
  long long need = (ntask + warps_per_block - 1) / warps_per_block;
  // persistent-style cap: enough resident blocks to fill every SM several times
  const long long cap = (long long)g_num_sms * (2048 / lc.block) * 4;
  if (need > cap) need = cap;
  return (int)(need < 1 ? 1 : need);
}

int launch_force(const Dev &d, const Box &b, const StepConsts &sc, const LaunchCfg &lc, int kick, int thermo,
                 int k, cudaStream_t st) {
  const int grid = force_grid_blocks(lc);
  if (grid > d.partials_blocks) return CAVGPU_E_ARG;  // each block writes its own partial sums
  int rc = lc.precision == CAVGPU_MIXED ? launch_tpa<true>(lc.tpa, kick, thermo != 0, grid, lc.block, d, b, sc, k, st)
                                        : launch_tpa<false>(lc.tpa, kick, thermo != 0, grid, lc.block, d, b, sc, k, st);
  if (rc) return rc;
  return cudaPeekAtLastError() == cudaSuccess ? CAVGPU_OK : CAVGPU_E_CUDA;
}

}  // namespace cav
