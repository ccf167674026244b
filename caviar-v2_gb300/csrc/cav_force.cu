// cav_force.cu -- the shifted-force LJ pair kernels (force_field::Lj::calculate_acceleration,
// src/force/lj.cpp:393-517), fused with the closing integrator update of the step.
//
// Full neighbour list, gather only (no atomics, deterministic): TPA lanes work on one
// atom, a warp on A = 32/TPA atoms, and the list layout (nbr_index) makes every
// iteration one coalesced 128-byte read of neighbour words.  Two precisions:
//   FP64  : image = x_j + s*L, all pair arithmetic in double;
//   MIXED : FP32 pair arithmetic on coordinates relative to each atom's build cell
//           (float4 x,y,z,type; cell offsets decoded from the stencil index), FP64
//           accumulation across lanes, FP64 acceleration/velocity/reductions.
#include <type_traits>

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
  double e6[MAXT * MAXT], e12[MAXT * MAXT];  // 6 eps4 and 12 eps4 (exact: products by 6 and 12)
  double minv[MAXT], mass[MAXT];
};
struct SmemTabF {
  float4 c4[MAXT * MAXT];  // {rc2, sig2, eps4, gc} of a type pair: one 128-bit load per pair
  float rc2[MAXT * MAXT], sig2[MAXT * MAXT], eps4[MAXT * MAXT], gc[MAXT * MAXT];
  float pk[MAXT * MAXT];   // 0.5 gc rc2 - uc, rounded once from FP64: V = eps4 s6 (s6 - 1) - 0.5 gc r2 + pk
  double minv[MAXT], mass[MAXT];
};
// per warp: the 27 image shifts s*L (FP64) or the cell widths (mixed) of the
// replica the warp's current atoms belong to (a warp never straddles two).  The
// mixed offsets are FP32 pairs d*wf + d*wlo: with the rounded width alone, every
// pair across a cell face would be displaced by the same d*(wf - w), a fixed
// distortion of the potential that changes pattern at each rebuild and drifts
// the NVE energy (measured -2.4e-4 per 1e6 steps).
template <bool MIXED>
struct WarpImages;
template <>
struct WarpImages<true> {
  float4 w;   // (wf, 0): cell widths rounded to FP32; a neighbour's offset is d*wf + d*wlo,
  float4 lo;  // (wlo, 0)  with d in {-1,0,1}^3 decoded from its stencil index
};

// Single-type systems keep the pair constants in registers (no table lookups).
struct OneType {
  float rc2, sig2, eps4, gc, pk;
};

// FP64 reciprocal by Newton-Raphson refinement of the hardware approximation
// (PTX rcp.approx.ftz.f64): each step y <- y + y (1 - x y) with two FMAs roughly
// doubles the correct bits (Markstein, "IA-64 and Elementary Functions", 2000), so
// two steps take the approximation to within an ulp or two of 1/x -- far inside the
// 1e-12 force tolerance -- at four FP64-pipe operations, the pipe this kernel is
// bound by.  Both orders of a pair see the same r^2, hence the same value.
__device__ __forceinline__ double rcp_nr(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  return fma(y, e, y);
}

// FP32 reciprocal from the hardware approximation (PTX rcp.approx.ftz.f32): one
// instruction instead of the correctly rounded sequence; it is a function of r^2
// alone, so both orders of a pair still see the same value.
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
template <>
struct WarpImages<false> {
  double3 v[27];
};

// Loads the pair table into shared memory (FP32 copy for the mixed form).
template <class Tab>
__device__ inline void load_tab(const Dev &d, Tab &tab) {
  const PairTab &T = *d.tab;
  const int nt = T.nt;
  for (int k = threadIdx.x; k < nt * nt; k += blockDim.x) {
    tab.rc2[k] = T.rc2[k]; tab.sig2[k] = T.sig2[k]; tab.eps4[k] = T.eps4[k]; tab.gc[k] = T.gc[k];
    if constexpr (std::is_same<Tab, SmemTabF>::value) {
      tab.c4[k] = make_float4(tab.rc2[k], tab.sig2[k], tab.eps4[k], tab.gc[k]);
      tab.pk[k] = (float)(0.5 * T.gc[k] * T.rc2[k] - T.uc[k]);
    } else {
      tab.uc[k] = T.uc[k];
      tab.e6[k] = 6.0 * T.eps4[k];
      tab.e12[k] = 12.0 * T.eps4[k];
    }
  }
  for (int k = threadIdx.x; k < nt; k += blockDim.x) { tab.minv[k] = T.minv[k]; tab.mass[k] = T.mass[k]; }
}

// Two FP32 values in one 64-bit register for the packed FP32x2 arithmetic of sm_100+
// (add/sub/mul/fma .rn.f32x2: each half rounded exactly as the scalar instruction).
struct F2 {
  unsigned long long v;
};
__device__ __forceinline__ F2 f2(float a, float b) {
  F2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void unf2(F2 x, float &a, float &b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x.v));
}
__device__ __forceinline__ F2 add2(F2 a, F2 b) {
  F2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 sub2(F2 a, F2 b) {
  F2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 mul2(F2 a, F2 b) {
  F2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
  F2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}

// A list chunk: read once per step and larger than L1, so it is not allocated in L1
// (which keeps the neighbour coordinates the gathers reuse).
__device__ __forceinline__ uint4 ld_list(const uint4 *p) {
  uint4 v;
  asm("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
      : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
      : "l"(p));
  return v;
}

// Mixed-form pair loop of one lane: list chunks t, t+TPA, ... of atom i (four words
// per 128-bit load; the next chunk's load and four neighbour coordinates in
// flight); `gather(word)` returns the neighbour's float4 (global memory or a
// shared-memory stage).  Two pairs go through each packed FP32x2 evaluation (even
// and odd list entries, with their own accumulators, folded at the end); a pair
// beyond its cutoff gets coef = 0.  ONE: single-type system, pair constants in
// registers; otherwise from the shared-memory table.
//
// ((r_j - r_i) + d wf) + d wlo, each sum rounded once (d wf and d wlo are exact
// products): rounding is symmetric under negation and i seen from j has offset -d,
// so d_ji = -d_ij bit for bit and the FP32 pair forces obey Newton's third law
// exactly (each half of a packed operation rounds as the scalar one).  d comes from
// the stencil index k = (dx+1) + 3 (dy+1) + 9 (dz+1) by integer arithmetic (a table
// in shared memory would load the L1 pipe that the neighbour gathers saturate).
template <int TPA, bool EV, bool ONE, class Gather>
__device__ __forceinline__ void mixed_pairs(const uint4 *row4, int nn, int t, const float4 ri, int ti, int nt,
                                            const SmemTabF &tab, const OneType c1, const float4 wf,
                                            const float4 wl, const float jtol, Gather gather, float &ax,
                                            float &ay, float &az, float &vr, float &pp) {
  F2 ax2 = f2(0.f, 0.f), ay2 = ax2, az2 = ax2, vr2 = ax2, pp2 = ax2;  // vr2: sum of +coef r^2
  uint4 nxt = 4 * t < nn ? ld_list(row4) : make_uint4(0, 0, 0, 0);
  for (int q = 0, k0 = 4 * t; k0 < nn; ++q, k0 += 4 * TPA) {
    const uint4 w4 = nxt;
    if (k0 + 4 * TPA < nn) nxt = ld_list(row4 + (size_t)(q + 1) * 32);  // the next list chunk in flight
    const uint32_t e[4] = {w4.x, w4.y, w4.z, w4.w};
    float4 rj[4];
#pragma unroll
    for (int u = 0; u < 4; ++u)  // four independent gathers in flight
      if (k0 + u < nn) rj[u] = gather(e[u]);
      else rj[u] = make_float4(1e18f, 1e18f, 1e18f, __int_as_float(ti));  // beyond every cutoff
#pragma unroll
    for (int a = 0; a < 4; a += 2) {
      if (k0 + a >= nn) break;
      // d = k - 1 for k in {0, 1, 2} without an int-to-float conversion: the float
      // with bits 0x4B400000 | k is 12582912 + k exactly, and 12582913 is subtracted
      float dd[6];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int code = e[a + h] >> CODE_SHIFT;
        const int kz = (code * 57) >> 9, r9 = code - 9 * kz, ky = (r9 * 11) >> 5, kx = r9 - 3 * ky;  // k/9, k/3
        dd[h] = __int_as_float(0x4B400000 | kx);
        dd[2 + h] = __int_as_float(0x4B400000 | ky);
        dd[4 + h] = __int_as_float(0x4B400000 | kz);
      }
      const F2 magic = f2(12582913.0f, 12582913.0f);
      const F2 ddx = sub2(f2(dd[0], dd[1]), magic), ddy = sub2(f2(dd[2], dd[3]), magic),
               ddz = sub2(f2(dd[4], dd[5]), magic);
      const F2 dx = fma2(ddx, f2(wl.x, wl.x), fma2(ddx, f2(wf.x, wf.x), sub2(f2(rj[a].x, rj[a + 1].x), f2(ri.x, ri.x))));
      const F2 dy = fma2(ddy, f2(wl.y, wl.y), fma2(ddy, f2(wf.y, wf.y), sub2(f2(rj[a].y, rj[a + 1].y), f2(ri.y, ri.y))));
      const F2 dz = fma2(ddz, f2(wl.z, wl.z), fma2(ddz, f2(wf.z, wf.z), sub2(f2(rj[a].z, rj[a + 1].z), f2(ri.z, ri.z))));
      const F2 r2d = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
      float r2a, r2b;
      unf2(r2d, r2a, r2b);
      float rc2a, rc2b, sg2a, sg2b, e4a, e4b, gca, gcb, pka, pkb;
      if (ONE) {
        rc2a = rc2b = c1.rc2; sg2a = sg2b = c1.sig2; e4a = e4b = c1.eps4; gca = gcb = c1.gc; pka = pkb = c1.pk;
      } else {
        const int ta = ti * nt + __float_as_int(rj[a].w), tb = ti * nt + __float_as_int(rj[a + 1].w);
        const float4 pa = tab.c4[ta], pb = tab.c4[tb];
        rc2a = pa.x; sg2a = pa.y; e4a = pa.z; gca = pa.w;
        rc2b = pb.x; sg2b = pb.y; e4b = pb.z; gcb = pb.w;
        pka = EV ? tab.pk[ta] : 0.0f;
        pkb = EV ? tab.pk[tb] : 0.0f;
      }
      const bool ina = r2a <= rc2a, inb = r2b <= rc2b;
      if (!(ina || inb)) continue;
      const float r2ca = fmaxf(r2a, jtol), r2cb = fmaxf(r2b, jtol);  // Lj jump_fix floor (0 when off)
      const F2 r2 = f2(r2ca, r2cb), r2i = f2(rcp_approx(r2ca), rcp_approx(r2cb));
      const F2 eps4 = f2(e4a, e4b);
      const F2 s2 = mul2(f2(sg2a, sg2b), r2i);
      const F2 s6 = mul2(mul2(s2, s2), s2);
      const F2 w = mul2(mul2(eps4, r2i), s6);
      F2 coef = fma2(w, fma2(f2(-12.0f, -12.0f), s6, f2(6.0f, 6.0f)), f2(-gca, -gcb));
      float ca, cb;
      unf2(coef, ca, cb);
      ca = ina ? ca : 0.0f;
      cb = inb ? cb : 0.0f;
      coef = f2(ca, cb);
      ax2 = fma2(coef, dx, ax2);
      ay2 = fma2(coef, dy, ay2);
      az2 = fma2(coef, dz, az2);
      if (EV) {
        vr2 = fma2(coef, r2, vr2);
        const F2 pe = fma2(mul2(eps4, s6), sub2(s6, f2(1.0f, 1.0f)),
                           fma2(f2(-0.5f * gca, -0.5f * gcb), r2, f2(pka, pkb)));
        float pa, pb;
        unf2(pe, pa, pb);
        pp2 = add2(pp2, f2(ina ? pa : 0.0f, inb ? pb : 0.0f));
      }
    }
  }
  float lo, hi;
  unf2(ax2, lo, hi); ax += lo + hi;
  unf2(ay2, lo, hi); ay += lo + hi;
  unf2(az2, lo, hi); az += lo + hi;
  if (EV) {
    unf2(vr2, lo, hi); vr -= lo + hi;
    unf2(pp2, lo, hi); pp += lo + hi;
  }
}

__device__ inline OneType one_type(const SmemTabF &tab) {
  return OneType{tab.rc2[0], tab.sig2[0], tab.eps4[0], tab.gc[0], tab.pk[0]};
}

// Folds the TPA lanes of each atom (lanes a, a+A, a+2A, ...; every lane of the warp
// calls this) and applies the closing update of the step to atom i on lane t == 0.
// KICK: 0 = store the acceleration only; 1 = velocity-Verlet closing kick
// v += (a + a_old) * (0.5 dt) (src/md_simulator.cpp:672-679); 2 = Langevin closing
// update v = (v a_L + eta b) + (a*0.5) dt (src/md_simulator.cpp:853-862).
// EV: accumulate virial, potential energy and KE (KICK == 2: the KE of the
// velocities at the end of the step, kept apart from the mid-step temperature's);
// batches also store virial and PE per slot for the per-replica folds.
// fuse: then the first half of the next step, with the arithmetic of the drift
// kernels (k_drift_vv, k_drift_lf, k_lang_a): the NaN check of the new acceleration,
// the drift, the half-skin test; the new coordinates go to the alternate buffer
// (FP64: pos_alt, which the neighbours of this step no longer read; mixed: rel_alt,
// the FP64 positions being this atom's alone).  Leap-frog keeps a_old = 0 for the
// next kick, as its drift kernel does.
template <int A, bool MIXED, int KICK, bool EV, class Tab>
__device__ __forceinline__ void finish_atom(const Dev &d, const Box &b, const StepConsts &sc, const Tab &tab,
                                            bool act, int t, int i, int ti, int rep, long long step, int fuse,
                                            double fx, double fy, double fz, double vir, double pe,
                                            double (&ke_p)[4], double (&ev_p)[2]) {
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
  if (!(act && t == 0)) return;
  const double mi = tab.minv[ti];
  dbl4 an = make_dbl4(fx * mi, fy * mi, fz * mi, 0.0);
  dbl4 v;
  if (KICK == 0) {
    d.acc[i] = an;
    if (EV) {
      v = d.vel[i];
      const double m = tab.mass[ti];
      ke_p[0] += m * (v.x * v.x + v.y * v.y + v.z * v.z);
      ke_p[1] += m * v.x; ke_p[2] += m * v.y; ke_p[3] += m * v.z;
    }
  } else if (KICK == 1) {
    v = d.vel[i];
    const dbl4 ao = d.acc[i];  // a(t), still in place until the store below
    if (MIXED) {
      v.x = fma(an.x + ao.x, sc.hdt, v.x);
      v.y = fma(an.y + ao.y, sc.hdt, v.y);
      v.z = fma(an.z + ao.z, sc.hdt, v.z);
    } else {  // v += (a + a_old) * (0.5 dt), the reference's order
      v.x = __dadd_rn(v.x, __dmul_rn(__dadd_rn(an.x, ao.x), sc.hdt));
      v.y = __dadd_rn(v.y, __dmul_rn(__dadd_rn(an.y, ao.y), sc.hdt));
      v.z = __dadd_rn(v.z, __dmul_rn(__dadd_rn(an.z, ao.z), sc.hdt));
    }
    if (EV) {
      const double m = tab.mass[ti];
      ke_p[0] += m * (v.x * v.x + v.y * v.y + v.z * v.z);
      ke_p[1] += m * v.x; ke_p[2] += m * v.y; ke_p[3] += m * v.z;
    }
  } else {
    v = d.vel[i];
    double e0 = 0.0, e1 = 0.0, e2 = 0.0;
    if (!sc.noise_off) {  // replica r draws the noise stream of seed + r with its local ids
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
    if (EV) {  // Atom_data::kinetic_energy() read after the step (the temperature was taken mid-step)
      const double m = tab.mass[ti];
      ke_p[0] += m * (v.x * v.x + v.y * v.y + v.z * v.z);
      ke_p[1] += m * v.x; ke_p[2] += m * v.y; ke_p[3] += m * v.z;
    }
  }
  if (KICK != 0) {
    if (fuse != FUSE_NONE) {  // the next step's first half (its drift kernel's arithmetic)
      nan_check(d, i, an);
      dbl4 x = d.pos[i];
      dbl4 ao = an;
      if (fuse == FUSE_VV) {
        drift_vv<MIXED>(x, v, an, sc);
      } else if (fuse == FUSE_LF) {
        drift_lf<MIXED>(x, v, an, sc);
        ao = make_dbl4(0.0, 0.0, 0.0, 0.0);  // a_old = 0 for the next kick
      } else {
        double e0 = 0.0, e1 = 0.0, e2 = 0.0;
        if (!sc.noise_off) {
          if (MIXED) langevin_eta_f(sc.seed + rep, step + 1, d.id[i], e0, e1, e2);
          else langevin_eta(sc.seed + rep, step + 1, d.id[i], e0, e1, e2);
        }
        lang_half<MIXED>(v, an, e0, e1, e2, sc);
        lang_move<MIXED>(x, v, sc);
      }
      d.acc[i] = ao;
      d.vel[i] = v;
      if (MIXED) {
        d.pos[i] = x;
        mixed_track(d, b, rep, i, x, d.rel_alt);
      } else {
        d.pos_alt[i] = x;
        half_skin_test(d, b, rep, i, x);
      }
    } else {
      d.acc[i] = an;
      d.vel[i] = v;
    }
  }
  if (EV) {
    ev_p[0] += vir;
    ev_p[1] += pe;
    if (d.ev_atom) d.ev_atom[i] = make_double2(vir, pe);
  }
}

// per-launch arguments of the pair kernels
struct ForceArgs {
  int k_in_chunk;                   // step index inside the chunk (Langevin noise counter)
  int fuse;                         // Fuse: the next step's drift in this launch
  int set_cond;                     // set `cond` at the end (inside a captured graph)
  cudaGraphConditionalHandle cond;  // the next step's rebuild node
  int fold;                         // the last block folds the thermo record (EV launches)
  FoldArgs fa;
};

// Sums of n blocks' partials of W doubles (W = 2 or 4) into v[0..W): thread t takes
// blocks t, t + B, t + 2B, ... in that order, four blocks' loads in flight at a time
// (L2 loads: other blocks wrote them).
template <int W>
__device__ __forceinline__ void fold_strided(const double *p, int n, double *v) {
  const int B = blockDim.x;
  for (int k0 = threadIdx.x; k0 < n; k0 += 4 * B) {
    double2 x[4][W / 2];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int h = 0; h < W / 2; ++h)
        x[u][h] = k0 + u * B < n ? __ldcg(reinterpret_cast<const double2 *>(p + (size_t)(k0 + u * B) * W) + h)
                                 : make_double2(0.0, 0.0);
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (k0 + u * B < n)
#pragma unroll
        for (int h = 0; h < W / 2; ++h) {
          v[2 * h] += x[u][h].x;
          v[2 * h + 1] += x[u][h].y;
        }
  }
}

// The thermo fold in the last block: every thread sums a strided subset of the
// partials, the block folds the threads' sums in a fixed order, thread 0 finishes
// the record.  The sums do not depend on which block finished last.
__device__ __noinline__ void fold_thermo(const Dev &d, const FoldArgs &fa, int nb_ev) {
  double v[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  fold_strided<4>(d.partials_ke, fa.nb_ke, v);
  fold_strided<2>(d.partials_ev, nb_ev, v + 4);
  fold_strided<4>(d.partials_ke_end, fa.nb_ke_end, v + 6);
  __shared__ double out[10];
  block_sum_store_f<10>(v, out);
  __syncthreads();
  if (threadIdx.x != 0) return;
  const ThermoCfg &tc = fa.tc;
  double res[5];
  const double P3[3] = {out[1], out[2], out[3]};
  thermo_finish(out[0], P3, d.thermo[5], out[4], out[5], tc.n, tc.n_r_df, tc.k_b, tc.volume, tc.langevin, res);
  if (fa.nb_ke_end > 0) {  // KE as Atom_data::kinetic_energy() reads it after the step
    double e[5];
    const double Q3[3] = {out[7], out[8], out[9]};
    thermo_finish(out[6], Q3, d.thermo[5], 0.0, 0.0, tc.n, tc.n_r_df, tc.k_b, tc.volume, tc.langevin, e);
    res[0] = e[0];
  }
#pragma unroll
  for (int q = 0; q < 5; ++q) d.thermo[q] = res[q];
  if (fa.ring_slot >= 0) {
    double *r = d.thermo_ring + (size_t)fa.ring_slot * THERMO_REC;
#pragma unroll
    for (int q = 0; q < THERMO_REC; ++q) r[q] = res[q];
  }
}

// End of a pair-kernel launch, every block: the last block to finish counts the
// step, turns a NaN seen by the fused drift into a halt, -- inside a graph -- sets
// the conditional node of the next step's rebuild, and (EV, fold) folds the thermo
// record unless the chunk halted.  The flag and partial stores of this launch are
// ordered before the ticket by the fence.
template <bool EV>
__device__ __forceinline__ void end_of_step(const Dev &d, bool was_halted, const ForceArgs &fa) {
  __shared__ int s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(d.force_ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __shared__ int s_fold;
  if (threadIdx.x == 0) {
    __threadfence();
    volatile int *f = d.flags;
    if (!was_halted) {
      f[F_STEPS_OK] = f[F_STEPS_OK] + 1;
      if (f[F_NAN]) f[F_HALT] = 1;
    }
    if (fa.set_cond) cudaGraphSetConditional(fa.cond, (f[F_REBUILD] != 0 && f[F_HALT] == 0) ? 1u : 0u);
    *d.force_ticket = 0u;
    s_fold = EV && fa.fold && f[F_HALT] == 0;
  }
  __syncthreads();
  if constexpr (EV) {
    if (s_fold) fold_thermo(d, fa.fa, gridDim.x);
  }
}

template <int KICK, bool EV>
__device__ inline void store_partials(const Dev &d, double (&ke_p)[4], double (&ev_p)[2]) {
  if (EV) {
    block_sum_store_f<2>(ev_p, &d.partials_ev[(size_t)blockIdx.x * 2]);
    __syncthreads();
    block_sum_store_f<4>(ke_p, &(KICK == 2 ? d.partials_ke_end : d.partials_ke)[(size_t)blockIdx.x * 4]);
  }
}

// Grid-strided pair kernel (the FP64 form; the mixed form when it has no segments):
// warp-sized tasks of A consecutive slots, neighbour coordinates gathered from
// global memory.
template <int TPA, bool MIXED, int KICK, bool EV, bool ONE>
__global__ void __launch_bounds__(256, MIXED ? 4 : 1) k_force(Dev d, Box b, StepConsts sc, ForceArgs fa) {
  constexpr int A = 32 / TPA;
  __shared__ typename std::conditional<MIXED, SmemTabF, SmemTabD>::type tab;
  __shared__ WarpImages<MIXED> wimg[8];
  __shared__ int s_halt;
  if (threadIdx.x == 0) s_halt = halted(d);
  load_tab(d, tab);
  __syncthreads();
  const bool was_halted = s_halt != 0;  // a step after a halt does nothing
  const int nt = d.tab->nt;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int a = lane % A, t = lane / A;
  const int n = sc.n, cap = d.cap;
  const int warps_total = (gridDim.x * blockDim.x) >> 5;
  const int ntask = was_halted ? 0 : (n + A - 1) / A;
  // EV: each thread's KE / virial / PE sums live in shared memory between tasks;
  // six doubles held in registers across the pair loop spill at 64 registers
  __shared__ double s_sum[EV ? 6 * 256 : 1];
  if (EV)
#pragma unroll
    for (int q = 0; q < 6; ++q) s_sum[q * 256 + threadIdx.x] = 0.0;
  long long step = 0;
  if (KICK == 2) step = *d.step_base + fa.k_in_chunk;
  int img_rep = -1;

  for (int task = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; task < ntask; task += warps_total) {
    const int rep = rep_of_slot(b, task * A);
    if (rep < 0) continue;  // a task of padding slots (uniform over the warp)
    if (rep != img_rep) {
      const RepBox &rb = repbox(b, rep);
      if constexpr (MIXED) {
        if (lane == 0) {
          wimg[wid].w = make_float4(rb.wf[0], rb.wf[1], rb.wf[2], 0.f);
          wimg[wid].lo = make_float4(rb.wlo[0], rb.wlo[1], rb.wlo[2], 0.f);
        }
      } else if (lane < 27) {
        const int sx = lane % 3 - 1, sy = (lane / 3) % 3 - 1, sz = lane / 9 - 1;
        wimg[wid].v[lane] = make_double3(sx * rb.L[0], sy * rb.L[1], sz * rb.L[2]);
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
        const float4 *rel = d.rel;
        mixed_pairs<TPA, EV, ONE>(row4, nn, t, ri, ti, nt, tab, one_type(tab), wimg[wid].w, wimg[wid].lo, sc.jump_tolf,
                             [rel](uint32_t w) { return __ldg(&rel[w & IDX_MASK]); }, ax, ay, az, vr, pp);
        fx = ax; fy = ay; fz = az; vir = vr; pe = pp;
      } else {
        const dbl4 xi = d.pos[i];
        ti = type_of(xi.w);
        const bool jump = sc.jump_tol > 0.0;
        // single type: the pair constants in registers, no table lookups; the cutoff
        // test r^2 <= rc^2 compares the bit patterns as integers (the same order for
        // doubles >= +0, and rc^2 < 0, an eps == 0 pair, admits none), off the FP64 pipe
        const int t1 = ti * nt;
        const long long rc2b1 = __double_as_longlong(tab.rc2[t1]);
        const double sig21 = tab.sig2[t1], e61 = tab.e6[t1], e121 = tab.e12[t1], gc1 = tab.gc[t1];
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
            // image x_j + s L (the reference's ghost coordinate); s = 0 for most
            // entries, where x_j + 0 is x_j exactly and the three adds are skipped
            const int code = (int)(e[u] >> CODE_SHIFT);
            double jx = xj[u].x, jy = xj[u].y, jz = xj[u].z;
            if (code != CODE_ZERO) {
              const double3 s = wimg[wid].v[code];
              jx += s.x; jy += s.y; jz += s.z;
            }
            const double dx = jx - xi.x, dy = jy - xi.y, dz = jz - xi.z;
            const double r2d = dx * dx + dy * dy + dz * dz;
            const int tt = ONE ? t1 : t1 + type_of(xj[u].w);
            const long long rc2b = ONE ? rc2b1 : __double_as_longlong(tab.rc2[tt]);
            if (__double_as_longlong(r2d) <= rc2b) {
              // Lj jump_fix (src/force/lj.cpp:459-468): r^2 floored at jump_tol after the
              // cutoff test (jump_tol = 0 when off); the direction stays dx, dy, dz
              double r2 = r2d;
              if (jump) r2 = r2d < sc.jump_tol ? sc.jump_tol : r2d;
              const double r2i = rcp_nr(r2);
              const double s2 = (ONE ? sig21 : tab.sig2[tt]) * r2i;
              const double s6 = s2 * s2 * s2;
              // eps4 s6 (6 - 12 s6) / r^2 - g(rc) as (s6 (e6 - e12 s6)) r2i - gc
              const double coef = ONE ? fma(s6 * fma(-e121, s6, e61), r2i, -gc1)
                                      : fma(s6 * fma(-tab.e12[tt], s6, tab.e6[tt]), r2i, -tab.gc[tt]);
              fx = fma(coef, dx, fx); fy = fma(coef, dy, fy); fz = fma(coef, dz, fz);
              if (EV) {
                vir -= coef * r2;
                pe += tab.eps4[tt] * (s6 * s6 - s6) - tab.uc[tt] - 0.5 * tab.gc[tt] * (r2 - tab.rc2[tt]);
              }
            }
          }
        }
      }
    }
    double ke_t[4] = {0.0, 0.0, 0.0, 0.0}, ev_t[2] = {0.0, 0.0};
    finish_atom<A, MIXED, KICK, EV>(d, b, sc, tab, act, t, i, ti, rep, step, fa.fuse, fx, fy, fz, vir, pe, ke_t,
                                    ev_t);
    if (EV) {
#pragma unroll
      for (int q = 0; q < 4; ++q) s_sum[q * 256 + threadIdx.x] += ke_t[q];
#pragma unroll
      for (int q = 0; q < 2; ++q) s_sum[(4 + q) * 256 + threadIdx.x] += ev_t[q];
    }
  }
  double ke_p[4] = {0.0, 0.0, 0.0, 0.0}, ev_p[2] = {0.0, 0.0};
  if (EV) {
#pragma unroll
    for (int q = 0; q < 4; ++q) ke_p[q] = s_sum[q * 256 + threadIdx.x];
#pragma unroll
    for (int q = 0; q < 2; ++q) ev_p[q] = s_sum[(4 + q) * 256 + threadIdx.x];
  }
  if (!was_halted) store_partials<KICK, EV>(d, ke_p, ev_p);
  if (KICK != 0) end_of_step<EV>(d, was_halted, fa);
}

// Mixed-form pair kernel over row segments.  A block takes a segment -- up to
// seg_umax - 2 consecutive cells of one x-row of one replica -- and stages into
// shared memory the FP32 coordinates of the atoms of the 9 neighbouring rows'
// cells x0-1 .. x0+len (periodic), so that every neighbour gather of the
// segment's atoms reads shared memory.  A list word (slot j, stencil index k)
// finds its copy through a table: row r = k / 3 of the stencil, staged cell
// u = (home cell - x0) + k % 3, index = j + (stage offset - first slot) of (r, u).
// The arithmetic is that of the grid-strided kernel, so results are the same bit
// for bit.  A segment whose stencil holds more atoms than the stage falls back to
// global gathers.  Warps take the segment's A-slot tasks; lanes whose atom lies
// outside the segment idle (their atoms belong to the adjacent segment).
template <int TPA, int KICK, bool EV, bool ONE>
__global__ void __launch_bounds__(256) k_force_seg(Dev d, Box b, StepConsts sc, ForceArgs fa) {
  constexpr int A = 32 / TPA;
  constexpr int AS = 5 - (TPA == 1 ? 0 : TPA == 2 ? 1 : TPA == 4 ? 2 : TPA == 8 ? 3 : 4);  // log2(A)
  __shared__ SmemTabF tab;
  __shared__ float4 s_wf, s_wl;
  __shared__ int s_total;
  extern __shared__ float4 stage[];
  const int umax = d.seg_umax;
  int *const toff = reinterpret_cast<int *>(stage + d.stage_cap);  // [9 * umax] stage offset - first slot
  int *const tcnt = toff + 9 * umax;                                 // [9 * umax] atoms, then exclusive scan
  __shared__ int s_halt;
  if (threadIdx.x == 0) s_halt = halted(d);
  load_tab(d, tab);
  __syncthreads();
  const bool was_halted = s_halt != 0;  // a step after a halt does nothing
  const int nt = d.tab->nt;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int a = lane % A, t = lane / A;
  const int cap = d.cap;
  double ke_p[4] = {0.0, 0.0, 0.0, 0.0};
  double ev_p[2] = {0.0, 0.0};
  long long step = 0;
  if (KICK == 2) step = *d.step_base + fa.k_in_chunk;
  int img_rep = -1;
  const int nseg = was_halted ? 0 : d.nseg;

  for (int sgi = blockIdx.x; sgi < nseg; sgi += gridDim.x) {
    const int4 sg = d.seg[sgi];
    const int rep = sg.x, cy = sg.y & 0xffff, cz = sg.y >> 16, x0 = sg.z, len = sg.w;
    const RepBox &rb = repbox(b, rep);
    const int U = len + 2, nq = 9 * U;
    __syncthreads();  // the previous segment's gathers are done with the stage and tables
    if (rep != img_rep) {
      if (threadIdx.x == 0) {
        s_wf = make_float4(rb.wf[0], rb.wf[1], rb.wf[2], 0.f);
        s_wl = make_float4(rb.wlo[0], rb.wlo[1], rb.wlo[2], 0.f);
      }
      img_rep = rep;
    }
    // staged cells q = r * U + u: row r = (dy + 1) + 3 (dz + 1), x cell x0 - 1 + u (periodic)
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
      const int r = q / U, u = q - r * U;
      int ny = cy + r % 3 - 1, nz = cz + r / 3 - 1, nx = (x0 - 1 + u) % rb.nc[0];
      if (nx < 0) nx += rb.nc[0];
      if (ny < 0) ny += rb.nc[1]; else if (ny >= rb.nc[1]) ny -= rb.nc[1];
      if (nz < 0) nz += rb.nc[2]; else if (nz >= rb.nc[2]) nz -= rb.nc[2];
      const int c = rb.cell_off + nx + rb.nc[0] * (ny + rb.nc[1] * nz);
      const int st = d.cell_start[c];
      toff[q] = st;
      tcnt[q] = d.cell_start[c + 1] - st;
    }
    __syncthreads();
    // exclusive scan of the counts (nq <= 9 * umax) by warp 0, 32 entries at a time
    if (wid == 0) {
      int carry = 0;
      for (int base = 0; base < nq; base += 32) {
        const int q = base + lane;
        const int v = q < nq ? tcnt[q] : 0;
        int inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(FULL_MASK, inc, o);
          if (lane >= o) inc += y;
        }
        if (q < nq) tcnt[q] = carry + inc - v;
        carry += __shfl_sync(FULL_MASK, inc, 31);
      }
      if (lane == 0) s_total = carry;
    }
    __syncthreads();
    const bool staged = s_total <= d.stage_cap;
    if (staged) {
      // copy: warp w takes staged cells w, w + nwarp, ...; lanes copy the cell's atoms
      for (int q = wid; q < nq; q += nwarp) {
        const int st = toff[q], base = tcnt[q];
        const int cn = (q + 1 < nq ? tcnt[q + 1] : s_total) - base;
        for (int k = lane; k < cn; k += 32) stage[base + k] = __ldg(&d.rel[st + k]);
      }
      __syncthreads();
      for (int q = threadIdx.x; q < nq; q += blockDim.x) toff[q] = tcnt[q] - toff[q];
    }
    __syncthreads();
    // the segment's atoms: slots of its cells (consecutive cell indices, so one range)
    const int rowc = rb.cell_off + rb.nc[0] * (cy + rb.nc[1] * cz);
    const int hs = d.cell_start[rowc + x0], he = d.cell_start[rowc + x0 + len];
    if (he > hs) {
      const int t_first = hs >> AS, t_last = (he - 1) >> AS;
      for (int task = t_first + wid; task <= t_last; task += nwarp) {
        const int i = task * A + a;
        const bool act = i >= hs && i < he;
        double fx = 0.0, fy = 0.0, fz = 0.0, vir = 0.0, pe = 0.0;
        int ti = 0;
        if (act) {
          const int nn = d.nnbr[i];
          const uint4 *row4 = reinterpret_cast<const uint4 *>(d.nbr + (size_t)task * cap * A) + (t * A + a);
          const float4 ri = d.rel[i];
          ti = __float_as_int(ri.w);
          float ax = 0.f, ay = 0.f, az = 0.f, vr = 0.f, pp = 0.f;
          if (staged) {
            const int hx = d.cell_of[i] - rowc - x0;  // home cell within the segment
            const int *tr = toff + hx;
            mixed_pairs<TPA, EV, ONE>(row4, nn, t, ri, ti, nt, tab, one_type(tab), s_wf, s_wl, sc.jump_tolf,
                                 [tr, U](uint32_t w) {  // `stage` is the block's shared array
                                   const int k = (int)(w >> CODE_SHIFT), r = (k * 11) >> 5;  // k / 3 for k < 27
                                   return stage[(int)(w & IDX_MASK) + tr[r * U + (k - 3 * r)]];
                                 },
                                 ax, ay, az, vr, pp);
          } else {
            const float4 *rel = d.rel;
            mixed_pairs<TPA, EV, ONE>(row4, nn, t, ri, ti, nt, tab, one_type(tab), s_wf, s_wl, sc.jump_tolf,
                                 [rel](uint32_t w) { return __ldg(&rel[w & IDX_MASK]); }, ax, ay, az, vr, pp);
          }
          fx = ax; fy = ay; fz = az; vir = vr; pe = pp;
        }
        finish_atom<A, true, KICK, EV>(d, b, sc, tab, act, t, i, ti, rep, step, fa.fuse, fx, fy, fz, vir, pe, ke_p,
                                       ev_p);
      }
    }
  }
  if (!was_halted) store_partials<KICK, EV>(d, ke_p, ev_p);
  if (KICK != 0) end_of_step<EV>(d, was_halted, fa);
}

template <int TPA, bool MIXED, int KICK>
static void launch_ev(bool ev, bool one, int grid, int block, const Dev &d, const Box &b, const StepConsts &sc,
                      const ForceArgs &fa, cudaStream_t st) {
  if (one) {  // single-type systems: pair constants in registers
    if (ev) k_force<TPA, MIXED, KICK, true, true><<<grid, block, 0, st>>>(d, b, sc, fa);
    else k_force<TPA, MIXED, KICK, false, true><<<grid, block, 0, st>>>(d, b, sc, fa);
    return;
  }
  if (ev) k_force<TPA, MIXED, KICK, true, false><<<grid, block, 0, st>>>(d, b, sc, fa);
  else k_force<TPA, MIXED, KICK, false, false><<<grid, block, 0, st>>>(d, b, sc, fa);
}

template <int TPA, bool MIXED>
static void launch_kick(int kick, bool ev, bool one, int grid, int block, const Dev &d, const Box &b,
                        const StepConsts &sc, const ForceArgs &fa, cudaStream_t st) {
  if (kick == 0) launch_ev<TPA, MIXED, 0>(ev, one, grid, block, d, b, sc, fa, st);
  else if (kick == 1) launch_ev<TPA, MIXED, 1>(ev, one, grid, block, d, b, sc, fa, st);
  else launch_ev<TPA, MIXED, 2>(ev, one, grid, block, d, b, sc, fa, st);
}

template <bool MIXED>
static int launch_tpa(int tpa, int kick, bool ev, bool one, int grid, int block, const Dev &d, const Box &b,
                      const StepConsts &sc, const ForceArgs &fa, cudaStream_t st) {
  switch (tpa) {
    case 1: launch_kick<1, MIXED>(kick, ev, one, grid, block, d, b, sc, fa, st); break;
    case 2: launch_kick<2, MIXED>(kick, ev, one, grid, block, d, b, sc, fa, st); break;
    case 4: launch_kick<4, MIXED>(kick, ev, one, grid, block, d, b, sc, fa, st); break;
    case 8: launch_kick<8, MIXED>(kick, ev, one, grid, block, d, b, sc, fa, st); break;
    case 16: launch_kick<16, MIXED>(kick, ev, one, grid, block, d, b, sc, fa, st); break;
    default: return CAVGPU_E_ARG;
  }
  return CAVGPU_OK;
}

// the segment kernel's variants, for launching and for their shared-memory attribute
template <int TPA, int KICK, bool EV>
static int seg_variant(bool launch, bool one, int grid, int block, size_t smem, const Dev &d, const Box &b,
                       const StepConsts &sc, const ForceArgs &fa, cudaStream_t st) {
  if (!launch) {
    if (cudaFuncSetAttribute(k_force_seg<TPA, KICK, EV, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess ||
        cudaFuncSetAttribute(k_force_seg<TPA, KICK, EV, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return CAVGPU_E_CUDA;
    return CAVGPU_OK;
  }
  if (one) k_force_seg<TPA, KICK, EV, true><<<grid, block, smem, st>>>(d, b, sc, fa);
  else k_force_seg<TPA, KICK, EV, false><<<grid, block, smem, st>>>(d, b, sc, fa);
  return CAVGPU_OK;
}
template <int TPA>
static int seg_kick(bool launch, int kick, bool ev, bool one, int grid, int block, size_t smem, const Dev &d,
                    const Box &b, const StepConsts &sc, const ForceArgs &fa, cudaStream_t st) {
  if (kick == 0) return ev ? seg_variant<TPA, 0, true>(launch, one, grid, block, smem, d, b, sc, fa, st)
                           : seg_variant<TPA, 0, false>(launch, one, grid, block, smem, d, b, sc, fa, st);
  if (kick == 1) return ev ? seg_variant<TPA, 1, true>(launch, one, grid, block, smem, d, b, sc, fa, st)
                           : seg_variant<TPA, 1, false>(launch, one, grid, block, smem, d, b, sc, fa, st);
  return ev ? seg_variant<TPA, 2, true>(launch, one, grid, block, smem, d, b, sc, fa, st)
            : seg_variant<TPA, 2, false>(launch, one, grid, block, smem, d, b, sc, fa, st);
}
static int seg_tpa(bool launch, int tpa, int kick, bool ev, bool one, int grid, int block, size_t smem,
                   const Dev &d, const Box &b, const StepConsts &sc, const ForceArgs &fa, cudaStream_t st) {
  switch (tpa) {
    case 1: return seg_kick<1>(launch, kick, ev, one, grid, block, smem, d, b, sc, fa, st);
    case 2: return seg_kick<2>(launch, kick, ev, one, grid, block, smem, d, b, sc, fa, st);
    case 4: return seg_kick<4>(launch, kick, ev, one, grid, block, smem, d, b, sc, fa, st);
    case 8: return seg_kick<8>(launch, kick, ev, one, grid, block, smem, d, b, sc, fa, st);
    case 16: return seg_kick<16>(launch, kick, ev, one, grid, block, smem, d, b, sc, fa, st);
    default: return CAVGPU_E_ARG;
  }
}

int prepare_force_seg(size_t smem_bytes) {
  Dev d{};
  Box b{};
  StepConsts sc{};
  for (int tpa = 1; tpa <= 16; tpa *= 2)
    for (int kick = 0; kick < 3; ++kick)
      for (int ev = 0; ev < 2; ++ev) {
        const int rc = seg_tpa(false, tpa, kick, ev != 0, false, 0, 0, smem_bytes, d, b, sc, ForceArgs{}, nullptr);
        if (rc) return rc;
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
  if (lc.precision == CAVGPU_MIXED && lc.use_seg && lc.nseg > 0)  // one segment per block at a time
    return lc.nseg < g_num_sms * 4 ? lc.nseg : g_num_sms * 4;
  const int A = 32 / lc.tpa;
  const long long ntask = (lc.n + A - 1) / A;
  const long long warps_per_block = lc.block / 32;
  long long need = (ntask + warps_per_block - 1) / warps_per_block;
  // the mixed kernels (64 registers) hold 32 warps per SM: one wave of resident blocks,
  // each warp walking its tasks grid-strided (fewer, longer-lived blocks: fewer block
  // reductions and tails; 5% less pair-kernel time and 16% less for the thermo
  // variant on the 1M-atom fluid than four waves); the FP64 kernels: four waves
  const long long cap = lc.precision == CAVGPU_MIXED ? (long long)g_num_sms * (1024 / lc.block)
                                                     : (long long)g_num_sms * (2048 / lc.block) * 4;
  if (need > cap) need = cap;
  return (int)(need < 1 ? 1 : need);
}

int launch_force(const Dev &d, const Box &b, const StepConsts &sc, const LaunchCfg &lc, int kick, int thermo,
                 int k, int fuse, int set_cond, cudaGraphConditionalHandle cond, cudaStream_t st,
                 const FoldArgs *fold) {
  const int grid = force_grid_blocks(lc);
  if (grid > d.partials_blocks) return CAVGPU_E_ARG;  // each block writes its own partial sums
  if (kick == 0 && (fuse || set_cond)) return CAVGPU_E_ARG;
  if (fold && (kick == 0 || !thermo)) return CAVGPU_E_ARG;  // the fold needs this launch's EV partials
  ForceArgs fa{k, fuse, set_cond, cond, fold ? 1 : 0, {}};
  if (fold) fa.fa = *fold;
  int rc;
  if (lc.precision == CAVGPU_MIXED && lc.use_seg && lc.nseg > 0) {
    if (!d.seg || d.nseg != lc.nseg) return CAVGPU_E_ARG;
    rc = seg_tpa(true, lc.tpa, kick, thermo != 0, lc.ntypes == 1, grid, lc.block,
                 seg_smem_bytes(d.stage_cap, d.seg_umax), d, b, sc, fa, st);
  } else {
    const bool one = lc.ntypes == 1;
    rc = lc.precision == CAVGPU_MIXED
             ? launch_tpa<true>(lc.tpa, kick, thermo != 0, one, grid, lc.block, d, b, sc, fa, st)
             : launch_tpa<false>(lc.tpa, kick, thermo != 0, one, grid, lc.block, d, b, sc, fa, st);
  }
  if (rc) return rc;
  return cudaPeekAtLastError() == cudaSuccess ? CAVGPU_OK : CAVGPU_E_CUDA;
}

}  // namespace cav
