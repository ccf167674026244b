// cav_force.cu -- the shifted-force LJ pair kernels (force_field::Lj::calculate_acceleration,
// src/force/lj.cpp:393-517), fused with the closing integrator update of the step.
//
// Full neighbour list, gather only (no atomics, deterministic): TPA lanes work on one
// atom, a warp on A = 32/TPA atoms.  The 32 slots of a window share a table of their
// distinct neighbours, and an atom's list entries are 16-bit indices into it; the
// list layout (nbr_index) makes every iteration one coalesced 512-byte read of eight
// entries per lane.  Two precisions:
//   FP64  : image = x_j + s*L, all pair arithmetic in double;
//   MIXED : FP32 pair arithmetic on coordinates relative to each atom's build cell
//           (float4 x,y,z,type; cell offsets from the entry and the table word), FP64
//           accumulation across lanes, FP64 acceleration/velocity/reductions.
#include <mutex>
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

// Bits a mixed-form neighbour coordinate carries in .w besides its type (< 256):
// ky << 8 | kz << 10, ky = dy+1 and kz = dz+1 of its cell relative to the atom's,
// from the table word's row r = ky + 3 kz ((11 r) >> 5 = r / 3 for r <= 8).
__device__ __forceinline__ int row_bits(uint32_t word) {
  const int r = (int)(word >> CODE_SHIFT), kz = (r * 11) >> 5;
  return ((r - 3 * kz) << 8) | (kz << 10);
}

// Mixed-form pair loop of one lane: list chunks t, t+TPA, ... of atom i (eight 16-bit
// entries per 128-bit load, the next chunk's load in flight), taken four entries at
// a time (four neighbour coordinates in flight); `gather(entry)` returns the
// neighbour's float4 with its row bits (a shared-memory stage of the window's table,
// or global memory through the table).  Two pairs go through each packed FP32x2
// evaluation (even and odd list entries, with their own accumulators, folded at the
// end); a pair beyond its cutoff gets coef = 0.  ONE: single-type system, pair
// constants in registers; otherwise from the shared-memory table.
//
// ((r_j - r_i) + d wf) + d wlo, each sum rounded once (d wf and d wlo are exact
// products): rounding is symmetric under negation and i seen from j has offset -d,
// so d_ji = -d_ij bit for bit and the FP32 pair forces obey Newton's third law
// exactly (each half of a packed operation rounds as the scalar one).  d = k - 1 per
// axis, kx from the entry, ky and kz from the coordinate's row bits.
template <int TPA, bool EV, bool ONE, class Gather>
__device__ __forceinline__ void mixed_pairs(const uint4 *row4, int nn, int t, const float4 ri, int ti, int nt,
                                            const SmemTabF &tab, const OneType c1, const float4 wf,
                                            const float4 wl, const float jtol, Gather gather, float &ax,
                                            float &ay, float &az, float &vr, float &pp) {
  F2 ax2 = f2(0.f, 0.f), ay2 = ax2, az2 = ax2, vr2 = ax2, pp2 = ax2;  // vr2: sum of +coef r^2
  uint4 nxt = 8 * t < nn ? ld_list(row4) : make_uint4(0, 0, 0, 0);
  for (int q = 0, k0 = 8 * t; k0 < nn; ++q, k0 += 8 * TPA) {
    const uint4 w4 = nxt;
    if (k0 + 8 * TPA < nn) nxt = ld_list(row4 + (size_t)(q + 1) * 32);  // the next list chunk in flight
    const uint32_t ew[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
    for (int hq = 0; hq < 2; ++hq) {
      const int kb = k0 + 4 * hq;
      if (kb >= nn) break;
      const uint32_t e[4] = {ew[2 * hq] & 0xffffu, ew[2 * hq] >> 16, ew[2 * hq + 1] & 0xffffu, ew[2 * hq + 1] >> 16};
      float4 rj[4];
#pragma unroll
      for (int u = 0; u < 4; ++u)  // four independent gathers in flight
        if (kb + u < nn) rj[u] = gather(e[u]);
        else rj[u] = make_float4(1e18f, 1e18f, 1e18f, __int_as_float(ti));  // beyond every cutoff
#pragma unroll
      for (int a = 0; a < 4; a += 2) {
        if (kb + a >= nn) break;
        // d = k - 1 for k in {0, 1, 2} without an int-to-float conversion: the float
        // with bits 0x4B400000 | k is 12582912 + k exactly, and 12582913 is subtracted
        float dd[6];
        int tj[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int wb = __float_as_int(rj[a + h].w);
          dd[h] = __int_as_float(0x4B400000 | (int)(e[a + h] >> TAB_BITS));
          dd[2 + h] = __int_as_float(0x4B400000 | ((wb >> 8) & 3));
          dd[4 + h] = __int_as_float(0x4B400000 | ((wb >> 10) & 3));
          tj[h] = wb & 0xff;
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
          const int ta = ti * nt + tj[0], tb = ti * nt + tj[1];
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

// End of a pair-kernel launch, every block: the last block to finish counts the
// step, turns a NaN seen by the fused drift into a halt, and -- inside a graph --
// sets the conditional node of the next step's rebuild.  The flag stores of this
// launch are ordered before the ticket by the fence.
__device__ __forceinline__ void end_of_step(const Dev &d, bool was_halted, int set_cond,
                                            cudaGraphConditionalHandle cond) {
  __syncthreads();
  if (threadIdx.x != 0) return;
  __threadfence();
  const unsigned int t = atomicAdd(d.force_ticket, 1u);
  if (t != gridDim.x - 1) return;
  __threadfence();
  volatile int *f = d.flags;
  if (!was_halted) {
    f[F_STEPS_OK] = f[F_STEPS_OK] + 1;
    if (f[F_NAN]) f[F_HALT] = 1;
  }
  if (set_cond) cudaGraphSetConditional(cond, (f[F_REBUILD] != 0 && f[F_HALT] == 0) ? 1u : 0u);
  *d.force_ticket = 0u;
}

// per-launch arguments of the pair kernels
struct ForceArgs {
  int k_in_chunk;                   // step index inside the chunk (Langevin noise counter)
  int fuse;                         // Fuse: the next step's drift in this launch
  int set_cond;                     // set `cond` at the end (inside a captured graph)
  cudaGraphConditionalHandle cond;  // the next step's rebuild node
  int scap;                         // MODE 2: window-table entries the stage of a warp holds
};

template <int KICK, bool EV>
__device__ inline void store_partials(const Dev &d, double (&ke_p)[4], double (&ev_p)[2]) {
  if (EV) {
    block_sum_store_f<2>(ev_p, &d.partials_ev[(size_t)blockIdx.x * 2]);
    __syncthreads();
    block_sum_store_f<4>(ke_p, &(KICK == 2 ? d.partials_ke_end : d.partials_ke)[(size_t)blockIdx.x * 4]);
  }
}

// Pair kernel.  Warps take windows of 32 slots (a window's table serves its atoms),
// each window as TPA tasks of A consecutive slots (the list layout's unit).
//   MODE 0: FP64, neighbour positions gathered from global memory through the table;
//   MODE 1: mixed, neighbour coordinates gathered from global memory through the table;
//   MODE 2: mixed, the window's table staged into shared memory first (fa.scap float4
//           per warp, dynamic): one coalesced read of the table, one gather per
//           distinct neighbour, and the pair loop reads shared memory; a window whose
//           table is longer than the stage gathers as MODE 1 does.
template <int TPA, int MODE, int KICK, bool EV, bool ONE>
__global__ void __launch_bounds__(256, MODE != 0 ? 4 : 1) k_force(Dev d, Box b, StepConsts sc, ForceArgs fa) {
  constexpr bool MIXED = MODE != 0, STAGED = MODE == 2;
  constexpr int A = 32 / TPA;
  extern __shared__ float4 stage_all[];
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
  const int n = sc.n, cap = d.cap, tcap = d.tcap;
  const int warps_total = (gridDim.x * blockDim.x) >> 5;
  const int nwin = was_halted ? 0 : (n + 31) >> 5;
  // EV: each thread's KE / virial / PE sums live in shared memory between tasks;
  // six doubles held in registers across the pair loop spill at 64 registers
  __shared__ double s_sum[EV ? 6 * 256 : 1];
  if (EV)
#pragma unroll
    for (int q = 0; q < 6; ++q) s_sum[q * 256 + threadIdx.x] = 0.0;
  long long step = 0;
  if (KICK == 2) step = *d.step_base + fa.k_in_chunk;
  int img_rep = -1;
  float4 *sm = stage_all + (size_t)wid * fa.scap;

  for (int win = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; win < nwin; win += warps_total) {
    const int rep = rep_of_slot(b, win << 5);  // a window lies in one replica; its first slot is an atom
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
    const uint32_t *wt = d.wtab + (size_t)win * tcap;
    bool staged = false;
    if constexpr (STAGED) {
      // the table's coordinates (current rel, row bits added), eight loads per lane in flight
      const int len = d.wtab_len[win];
      staged = len <= fa.scap;
      for (int k0 = 0; staged && k0 < len; k0 += 256) {
        uint32_t w[8];
        float4 r[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int k = k0 + 32 * u + lane;
          w[u] = k < len ? __ldg(wt + k) : 0u;  // slot 0 stands in past the end
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) r[u] = __ldg(&d.rel[w[u] & IDX_MASK]);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int k = k0 + 32 * u + lane;
          if (k < len) {
            r[u].w = __int_as_float(__float_as_int(r[u].w) | row_bits(w[u]));
            sm[k] = r[u];
          }
        }
      }
      __syncwarp();
    }
    for (int s = 0; s < TPA; ++s) {
      const int task = win * TPA + s;
      const int i = task * A + a;
      const bool act = i < n && rep_of_slot(b, i) >= 0;
      double fx = 0.0, fy = 0.0, fz = 0.0, vir = 0.0, pe = 0.0;
      int ti = 0;
      if (act) {
        const int nn = d.nnbr[i];
        // this lane's list entries: chunk g = t + TPA q (entries 8g..8g+7), one 128-bit
        // load each; the warp's loads for one q cover 512 consecutive bytes (nbr_index)
        const uint4 *row4 = reinterpret_cast<const uint4 *>(d.nbr + (size_t)task * cap * A) + (t * A + a);
        if constexpr (MIXED) {
          const float4 ri = d.rel[i];
          ti = __float_as_int(ri.w);
          float ax = 0.f, ay = 0.f, az = 0.f, vr = 0.f, pp = 0.f;
          if (STAGED && staged) {
            mixed_pairs<TPA, EV, ONE>(row4, nn, t, ri, ti, nt, tab, one_type(tab), wimg[wid].w, wimg[wid].lo,
                                      sc.jump_tolf, [sm](uint32_t e) { return sm[e & TAB_IDX_MASK]; }, ax, ay, az,
                                      vr, pp);
          } else {
            const float4 *rel = d.rel;
            mixed_pairs<TPA, EV, ONE>(row4, nn, t, ri, ti, nt, tab, one_type(tab), wimg[wid].w, wimg[wid].lo,
                                      sc.jump_tolf,
                                      [wt, rel](uint32_t e) {
                                        const uint32_t w = __ldg(wt + (e & TAB_IDX_MASK));
                                        float4 r = __ldg(&rel[w & IDX_MASK]);
                                        r.w = __int_as_float(__float_as_int(r.w) | row_bits(w));
                                        return r;
                                      },
                                      ax, ay, az, vr, pp);
          }
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
          for (int q = 0, k0 = 8 * t; k0 < nn; ++q, k0 += 8 * TPA) {
            const uint4 w4 = __ldg(row4 + (size_t)q * 32);
            const uint32_t ew[4] = {w4.x, w4.y, w4.z, w4.w};
            // the table words, then the positions: eight independent gathers in flight
            uint32_t wd[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const uint32_t e = (ew[u >> 1] >> (16 * (u & 1))) & 0xffffu;
              wd[u] = k0 + u < nn ? __ldg(wt + (e & TAB_IDX_MASK)) : 0u;
            }
            dbl4 xj[8];
#pragma unroll
            for (int u = 0; u < 8; ++u)
              if (k0 + u < nn) xj[u] = ldg_dbl4(&d.pos[wd[u] & IDX_MASK]);
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              if (k0 + u >= nn) break;
              // image x_j + s L (the reference's ghost coordinate); s = 0 for most
              // entries, where x_j + 0 is x_j exactly and the three adds are skipped
              const int code = (int)(wd[u] >> CODE_SHIFT);
              double jx = xj[u].x, jy = xj[u].y, jz = xj[u].z;
              if (code != CODE_ZERO) {
                const double3 sh = wimg[wid].v[code];
                jx += sh.x; jy += sh.y; jz += sh.z;
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
    if constexpr (STAGED) __syncwarp();  // the stage is refilled for the next window
  }
  double ke_p[4] = {0.0, 0.0, 0.0, 0.0}, ev_p[2] = {0.0, 0.0};
  if (EV) {
#pragma unroll
    for (int q = 0; q < 4; ++q) ke_p[q] = s_sum[q * 256 + threadIdx.x];
#pragma unroll
    for (int q = 0; q < 2; ++q) ev_p[q] = s_sum[(4 + q) * 256 + threadIdx.x];
  }
  if (!was_halted) store_partials<KICK, EV>(d, ke_p, ev_p);
  if (KICK != 0) end_of_step(d, was_halted, fa.set_cond, fa.cond);
}

// Launch (or, with launch = false, raise the dynamic shared-memory limit of) one variant.
template <int TPA, int MODE, int KICK>
static int launch_ev(bool launch, bool ev, bool one, int grid, int block, size_t smem, const Dev &d, const Box &b,
                     const StepConsts &sc, const ForceArgs &fa, cudaStream_t st) {
  auto k = one ? (ev ? k_force<TPA, MODE, KICK, true, true> : k_force<TPA, MODE, KICK, false, true>)
               : (ev ? k_force<TPA, MODE, KICK, true, false> : k_force<TPA, MODE, KICK, false, false>);
  if (!launch)
    return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FORCE_SMEM_MAX) == cudaSuccess
               ? CAVGPU_OK
               : CAVGPU_E_CUDA;
  k<<<grid, block, smem, st>>>(d, b, sc, fa);
  return CAVGPU_OK;
}

template <int TPA, int MODE>
static int launch_kick(bool launch, int kick, bool ev, bool one, int grid, int block, size_t smem, const Dev &d,
                       const Box &b, const StepConsts &sc, const ForceArgs &fa, cudaStream_t st) {
  if (kick == 0) return launch_ev<TPA, MODE, 0>(launch, ev, one, grid, block, smem, d, b, sc, fa, st);
  if (kick == 1) return launch_ev<TPA, MODE, 1>(launch, ev, one, grid, block, smem, d, b, sc, fa, st);
  return launch_ev<TPA, MODE, 2>(launch, ev, one, grid, block, smem, d, b, sc, fa, st);
}

template <int MODE>
static int launch_tpa(bool launch, int tpa, int kick, bool ev, bool one, int grid, int block, size_t smem,
                      const Dev &d, const Box &b, const StepConsts &sc, const ForceArgs &fa, cudaStream_t st) {
  switch (tpa) {
    case 1: return launch_kick<1, MODE>(launch, kick, ev, one, grid, block, smem, d, b, sc, fa, st);
    case 2: return launch_kick<2, MODE>(launch, kick, ev, one, grid, block, smem, d, b, sc, fa, st);
    case 4: return launch_kick<4, MODE>(launch, kick, ev, one, grid, block, smem, d, b, sc, fa, st);
    case 8: return launch_kick<8, MODE>(launch, kick, ev, one, grid, block, smem, d, b, sc, fa, st);
    case 16: return launch_kick<16, MODE>(launch, kick, ev, one, grid, block, smem, d, b, sc, fa, st);
    default: return CAVGPU_E_ARG;
  }
}

int prepare_force() {
  static std::once_flag once;
  static int rc = CAVGPU_OK;
  std::call_once(once, [] {
    const Dev d{};
    const Box b{};
    const StepConsts sc{};
    for (int tpa = 1; tpa <= 16 && !rc; tpa *= 2)
      for (int kick = 0; kick < 3 && !rc; ++kick)
        for (int v = 0; v < 4 && !rc; ++v)
          rc = launch_tpa<2>(false, tpa, kick, v & 1, v >> 1, 0, 0, 0, d, b, sc, ForceArgs{}, nullptr);
  });
  return rc;
}

static int g_num_sms = 0;

int force_grid_blocks(const LaunchCfg &lc) {
  if (!g_num_sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 148;
  }
  const long long nwin = (lc.n + 31) / 32;
  const long long warps_per_block = lc.block / 32;
  long long need = (nwin + warps_per_block - 1) / warps_per_block;
  // persistent-style cap: enough resident blocks to fill every SM several times
  const long long cap = (long long)g_num_sms * (2048 / lc.block) * 4;
  if (need > cap) need = cap;
  return (int)(need < 1 ? 1 : need);
}

int launch_force(const Dev &d, const Box &b, const StepConsts &sc, const LaunchCfg &lc, int kick, int thermo,
                 int k, int fuse, int set_cond, cudaGraphConditionalHandle cond, cudaStream_t st) {
  const int grid = force_grid_blocks(lc);
  if (grid > d.partials_blocks) return CAVGPU_E_ARG;  // each block writes its own partial sums
  if (kick == 0 && (fuse || set_cond)) return CAVGPU_E_ARG;
  if (lc.tcap != d.tcap) return CAVGPU_E_ARG;
  const bool staged = force_staged(lc);
  const ForceArgs fa{k, fuse, set_cond, cond, staged ? lc.scap : 0};
  const bool one = lc.ntypes == 1, ev = thermo != 0;
  int rc;
  if (lc.precision != CAVGPU_MIXED)
    rc = launch_tpa<0>(true, lc.tpa, kick, ev, one, grid, lc.block, 0, d, b, sc, fa, st);
  else if (staged)
    rc = launch_tpa<2>(true, lc.tpa, kick, ev, one, grid, lc.block, force_smem_bytes(lc.block, lc.scap), d, b, sc,
                       fa, st);
  else
    rc = launch_tpa<1>(true, lc.tpa, kick, ev, one, grid, lc.block, 0, d, b, sc, fa, st);
  if (rc) return rc;
  return cudaPeekAtLastError() == cudaSuccess ? CAVGPU_OK : CAVGPU_E_CUDA;
}

}  // namespace cav
