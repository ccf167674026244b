/*
 * cav_oracle.c -- CPU restatement of CAVIAR2's MD step (test infrastructure).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * this file; the shipped GPU library never links it.  Every function names
 * the reference lines it restates.  Loop orders and floating-point expression
 * orders follow the reference so that, compiled with -ffp-contract=off, the
 * outputs equal the reference's bit for bit (checked against fixtures that
 * the reference itself produced; see tests/golden/make_golden.py).
 */
#include "cav_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* growable arrays                                                            */
/* ------------------------------------------------------------------------ */
typedef struct { int32_t *a; int64_t n, cap; } ivec;
typedef struct { double *a; int64_t n, cap; } dvec;

static int iv_push(ivec *v, int32_t x) {
  if (v->n == v->cap) {
    int64_t nc = v->cap ? v->cap * 2 : 64;
    int32_t *na = (int32_t *)realloc(v->a, (size_t)nc * sizeof(int32_t));
    if (!na) return -1;
    v->a = na; v->cap = nc;
  }
  v->a[v->n++] = x;
  return 0;
}
static int dv_push3(dvec *v, double x, double y, double z) {
  if (v->n + 3 > v->cap) {
    int64_t nc = v->cap ? v->cap * 2 : 192;
    while (nc < v->n + 3) nc *= 2;
    double *na = (double *)realloc(v->a, (size_t)nc * sizeof(double));
    if (!na) return -1;
    v->a = na; v->cap = nc;
  }
  v->a[v->n++] = x; v->a[v->n++] = y; v->a[v->n++] = z;
  return 0;
}

struct orc_sys {
  orc_params p;
  int32_t n;
  double *pos, *vel, *acc, *acc_old, *pos_old_nl;
  int32_t *type;
  int32_t *img;                /* Atom_struct::msd_domain_cross, x3 */
  int32_t *mol;                /* Atom_struct::molecule_index */
  unsigned char *in_domain;    /* Atom_struct::mpi_rank == my rank (src/atom_data.cpp:817-839) */
  /* Domain (src/domain.cpp:309-328, 495-502): single rank, nprocs = 1 */
  double size[3];              /* size_global = upper_global - lower_global */
  double lo_local[3], hi_local[3], size_local[3];
  /* ghosts (src/atom_data/exchange_ghost_single_md_domain.cpp) */
  dvec gpos;
  ivec gsrc, gshift;           /* source owned index; shift s (image = pos + s*L) x3 */
  dvec gpos_old_nl;
  int64_t ghost_old_n;
  /* Neighborlist */
  double cutoff_extra, threshold_sq, cutoff_inv;
  int32_t nb[3];
  int32_t *bin_start, *bin_count, *bin_items;   /* CSR binlist, insertion order */
  int32_t *nbin_n, *nbin;                        /* neigh_bin: per bin up to 27 bins */
  int64_t nl_start_cap;
  int64_t *nl_start;
  int32_t *nl_count;
  ivec nl;
  int64_t rebuilds;
  int built;
  /* thermo */
  double virial, pe, ke, temperature, pressure;
  int64_t current_step;
  int setup_done;
};

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 (J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw,        */
/* "Parallel random numbers: as easy as 1, 2, 3", SC'11): round function and  */
/* Weyl key schedule as published.                                            */
/* ------------------------------------------------------------------------ */
void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += W0; k1 += W1; }
    uint64_t p0 = (uint64_t)M0 * c0, p1 = (uint64_t)M1 * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

#define ORC_LANG_TAG 0x4C414E47u /* counter word 3 of the Langevin stream */

void orc_langevin_eta(uint64_t seed, uint64_t step, uint32_t id, double eta[3]) {
  uint32_t ctr[4] = {(uint32_t)step, (uint32_t)(step >> 32), id, ORC_LANG_TAG};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t r[4];
  orc_philox4x32_10(ctr, key, r);
  const double s = 2.3283064365386963e-10; /* 2^-32 */
  double u0 = ((double)r[0] + 0.5) * s, u1 = ((double)r[1] + 0.5) * s;
  double u2 = ((double)r[2] + 0.5) * s;
  /* Box-Muller: r = sqrt(-2 ln u), angle 2*pi*u' */
  double rad0 = sqrt(-2.0 * log(u0));
  double rad1 = sqrt(-2.0 * log(u2));
  const double two_pi = 6.283185307179586;
  eta[0] = rad0 * cos(two_pi * u1);
  eta[1] = rad0 * sin(two_pi * u1);
  double u3 = ((double)r[3] + 0.5) * s;
  eta[2] = rad1 * cos(two_pi * u3);
}

/* ------------------------------------------------------------------------ */
/* Domain::fix_position  (src/domain.cpp:443-493)                            */
/* ------------------------------------------------------------------------ */
static int fix_position(const orc_sys *s, double *p, int32_t *msd) {
  int wrapped = 0;
  for (int d = 0; d < 3; ++d) {
    if (s->p.bc[d] != 1) continue;
    if (p[d] < s->p.lo[d]) { wrapped = 1; p[d] += s->size[d]; msd[d] -= 1; }
    else if (p[d] > s->p.hi[d]) { wrapped = 1; p[d] -= s->size[d]; msd[d] += 1; }
  }
  return wrapped;
}

/* Atom_data::exchange_owned_single_md_domain
 * (src/atom_data/exchange_owned_single_md_domain.cpp:29-56); the crossings add
 * up in msd_domain_cross (kept whether or not msd_process is on) */
static int exchange_owned(orc_sys *s) {
  int upd = 0;
  for (int32_t i = 0; i < s->n; ++i)
    if (fix_position(s, &s->pos[3 * i], &s->img[3 * i])) upd = 1;
  return upd;
}

/* Atom_data::exchange_ghost_single_md_domain
 * (src/atom_data/exchange_ghost_single_md_domain.cpp:24-215): face, edge and
 * corner images emitted in the order x, y, z, xy, xz, yz, xyz. */
static int exchange_ghost(orc_sys *s) {
  s->gpos.n = 0; s->gsrc.n = 0; s->gshift.n = 0;
  const double gc = s->p.ghost_cutoff;
  const double x_llow = s->p.lo[0] + gc, x_lupp = s->p.hi[0] - gc;
  const double y_llow = s->p.lo[1] + gc, y_lupp = s->p.hi[1] - gc;
  const double z_llow = s->p.lo[2] + gc, z_lupp = s->p.hi[2] - gc;
  const double xw = s->size[0], yw = s->size[1], zw = s->size[2];
  for (int32_t i = 0; i < s->n; ++i) {
    const double *q = &s->pos[3 * i];
    int xv = q[0] < x_llow ? -1 : (q[0] > x_lupp ? 1 : 0);
    int yv = q[1] < y_llow ? -1 : (q[1] > y_lupp ? 1 : 0);
    int zv = q[2] < z_llow ? -1 : (q[2] > z_lupp ? 1 : 0);
    xv *= s->p.bc[0]; yv *= s->p.bc[1]; zv *= s->p.bc[2];
    /* image coordinate is pos - val*width, exactly as the reference */
    const double gx = q[0] - xv * xw, gy = q[1] - yv * yw, gz = q[2] - zv * zw;
    int combos[7][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
    for (int c = 0; c < 7; ++c) {
      int ux = combos[c][0], uy = combos[c][1], uz = combos[c][2];
      if ((ux && xv == 0) || (uy && yv == 0) || (uz && zv == 0)) continue;
      if (dv_push3(&s->gpos, ux ? gx : q[0], uy ? gy : q[1], uz ? gz : q[2])) return ORC_E_NOMEM;
      if (iv_push(&s->gsrc, i)) return ORC_E_NOMEM;
      if (iv_push(&s->gshift, ux ? -xv : 0) || iv_push(&s->gshift, uy ? -yv : 0) ||
          iv_push(&s->gshift, uz ? -zv : 0))
        return ORC_E_NOMEM;
    }
  }
  return ORC_OK;
}

static inline int32_t ghost_n(const orc_sys *s) { return (int32_t)(s->gpos.n / 3); }

/* ------------------------------------------------------------------------ */
/* Neighborlist                                                               */
/* ------------------------------------------------------------------------ */
/* Neighborlist::binlist_index (src/neighborlist.cpp:392-414) */
static void binlist_index(const orc_sys *s, const double *q, int32_t ind[3]) {
  for (int d = 0; d < 3; ++d) {
    int32_t v = (int32_t)floor((q[d] - s->lo_local[d]) * s->cutoff_inv);
    if (v < 0) v = 0;
    if (v >= s->nb[d]) v = s->nb[d] - 1;
    ind[d] = v;
  }
}

/* Neighborlist::make_neigh_bin (src/neighborlist.cpp:560-672): periodic
 * 27-stencil per bin, first occurrence kept by remove_duplicates. */
static int make_neigh_bin(orc_sys *s) {
  const int32_t nx = s->nb[0], ny = s->nb[1], nz = s->nb[2];
  const int64_t nbins = (int64_t)nx * ny * nz;
  free(s->nbin_n); free(s->nbin);
  s->nbin_n = (int32_t *)calloc((size_t)nbins, sizeof(int32_t));
  s->nbin = (int32_t *)malloc((size_t)nbins * 27 * 3 * sizeof(int32_t));
  if (!s->nbin_n || !s->nbin) return ORC_E_NOMEM;
  for (int32_t ix = 0; ix < nx; ++ix)
    for (int32_t iy = 0; iy < ny; ++iy)
      for (int32_t iz = 0; iz < nz; ++iz) {
        int32_t xmin = ix - 1, xmax = ix + 1, ymin = iy - 1, ymax = iy + 1, zmin = iz - 1, zmax = iz + 1;
        if (s->p.bc[0] == 0) { if (xmin == -1) xmin = 0; if (xmax == nx) xmax = nx - 1; }
        if (s->p.bc[1] == 0) { if (ymin == -1) ymin = 0; if (ymax == ny) ymax = ny - 1; }
        if (s->p.bc[2] == 0) { if (zmin == -1) zmin = 0; if (zmax == nz) zmax = nz - 1; }
        int64_t k = ix + (int64_t)nx * iy + (int64_t)nx * ny * iz;
        int32_t *lst = &s->nbin[k * 27 * 3];
        int32_t cnt = 0;
        for (int32_t a = xmin; a <= xmax; ++a)
          for (int32_t b = ymin; b <= ymax; ++b)
            for (int32_t c = zmin; c <= zmax; ++c) {
              int32_t v[3] = {a, b, c};
              if (v[0] == nx) v[0] = 0;
              if (v[1] == ny) v[1] = 0;
              if (v[2] == nz) v[2] = 0;
              if (v[0] == -1) v[0] = nx - 1;
              if (v[1] == -1) v[1] = ny - 1;
              if (v[2] == -1) v[2] = nz - 1;
              int dup = 0;
              for (int32_t e = 0; e < cnt; ++e)
                if (lst[3 * e] == v[0] && lst[3 * e + 1] == v[1] && lst[3 * e + 2] == v[2]) { dup = 1; break; }
              if (dup) continue;
              lst[3 * cnt] = v[0]; lst[3 * cnt + 1] = v[1]; lst[3 * cnt + 2] = v[2];
              ++cnt;
            }
        s->nbin_n[k] = cnt;
      }
  return ORC_OK;
}

/* Neighborlist::init (src/neighborlist.cpp:303-390).  The reference never
 * sets `initialized`, so update_is_needed() re-runs this on every call; the
 * restatement does the same work. */
static int nl_init(orc_sys *s) {
  s->cutoff_extra = s->p.nl_cutoff * s->p.nl_coef;
  s->threshold_sq = 0.25 * (s->cutoff_extra - s->p.nl_cutoff) * (s->cutoff_extra - s->p.nl_cutoff);
  if (!s->p.use_cell_list) return ORC_OK;
  s->cutoff_inv = 1.0 / s->cutoff_extra;
  int32_t nb[3];
  for (int d = 0; d < 3; ++d) nb[d] = (int32_t)ceil(s->size_local[d] * s->cutoff_inv);
  int changed = (nb[0] != s->nb[0] || nb[1] != s->nb[1] || nb[2] != s->nb[2] || !s->nbin);
  s->nb[0] = nb[0]; s->nb[1] = nb[1]; s->nb[2] = nb[2];
  if (changed) {
    free(s->bin_start); free(s->bin_count);
    int64_t nbins = (int64_t)nb[0] * nb[1] * nb[2];
    s->bin_start = (int32_t *)calloc((size_t)nbins + 1, sizeof(int32_t));
    s->bin_count = (int32_t *)calloc((size_t)nbins, sizeof(int32_t));
    if (!s->bin_start || !s->bin_count) return ORC_E_NOMEM;
  }
  return make_neigh_bin(s);
}

static inline int64_t bin_lin(const orc_sys *s, const int32_t ind[3]) {
  return ind[0] + (int64_t)s->nb[0] * ind[1] + (int64_t)s->nb[0] * s->nb[1] * ind[2];
}

/* Neighborlist::update_cell_list (src/neighborlist.cpp:422-455): owned atoms
 * then ghosts (index g + N), in insertion order per bin. */
static int update_cell_list(orc_sys *s) {
  const int64_t nbins = (int64_t)s->nb[0] * s->nb[1] * s->nb[2];
  const int32_t n = s->n, g = ghost_n(s);
  memset(s->bin_count, 0, (size_t)nbins * sizeof(int32_t));
  int32_t *which = (int32_t *)malloc(((size_t)n + g + 1) * sizeof(int32_t));
  if (!which) return ORC_E_NOMEM;
  int32_t ind[3];
  for (int32_t i = 0; i < n + g; ++i) {
    const double *q = i < n ? &s->pos[3 * i] : &s->gpos.a[3 * (i - n)];
    binlist_index(s, q, ind);
    which[i] = (int32_t)bin_lin(s, ind);
    s->bin_count[which[i]]++;
  }
  s->bin_start[0] = 0;
  for (int64_t b = 0; b < nbins; ++b) s->bin_start[b + 1] = s->bin_start[b] + s->bin_count[b];
  free(s->bin_items);
  s->bin_items = (int32_t *)malloc(((size_t)n + g + 1) * sizeof(int32_t));
  if (!s->bin_items) { free(which); return ORC_E_NOMEM; }
  memset(s->bin_count, 0, (size_t)nbins * sizeof(int32_t));
  for (int32_t i = 0; i < n + g; ++i) {
    int32_t b = which[i];
    s->bin_items[s->bin_start[b] + s->bin_count[b]++] = i;
  }
  free(which);
  return ORC_OK;
}

static int nl_reserve(orc_sys *s) {
  if (s->nl_start_cap < s->n) {
    free(s->nl_start); free(s->nl_count);
    s->nl_start = (int64_t *)malloc(((size_t)s->n + 1) * sizeof(int64_t));
    s->nl_count = (int32_t *)malloc(((size_t)s->n + 1) * sizeof(int32_t));
    if (!s->nl_start || !s->nl_count) return ORC_E_NOMEM;
    s->nl_start_cap = s->n;
  }
  s->nl.n = 0;
  return ORC_OK;
}

static void snapshot_old(orc_sys *s) {
  memcpy(s->pos_old_nl, s->pos, (size_t)s->n * 3 * sizeof(double));
  s->gpos_old_nl.n = 0;
  for (int64_t k = 0; k + 2 < s->gpos.n; k += 3)
    dv_push3(&s->gpos_old_nl, s->gpos.a[k], s->gpos.a[k + 1], s->gpos.a[k + 2]);
  s->ghost_old_n = ghost_n(s);
  s->rebuilds++;
  s->built = 1;
}

static inline double dist2(const double *a, const double *b) {
  /* (a - b) * (a - b) = x*x + y*y + z*z, left to right (vector3d.hpp:66-69) */
  double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
  return dx * dx + dy * dy + dz * dz;
}

/* Neighborlist::update_verlet_list (src/neighborlist.cpp:247-297) */
static int update_verlet_list(orc_sys *s) {
  if (nl_reserve(s)) return ORC_E_NOMEM;
  const double ce2 = s->cutoff_extra * s->cutoff_extra;
  const int32_t n = s->n, g = ghost_n(s);
  for (int32_t i = 0; i < n; ++i) {
    s->nl_start[i] = s->nl.n;
    const double *pi = &s->pos[3 * i];
    for (int32_t j = i + 1; j < n; ++j)
      if (dist2(&s->pos[3 * j], pi) < ce2 && iv_push(&s->nl, j)) return ORC_E_NOMEM;
    for (int32_t j = 0; j < g; ++j)
      if (dist2(&s->gpos.a[3 * j], pi) < ce2 && iv_push(&s->nl, j + n)) return ORC_E_NOMEM;
    s->nl_count[i] = (int32_t)(s->nl.n - s->nl_start[i]);
  }
  snapshot_old(s);
  return ORC_OK;
}

/* Neighborlist::update_verlet_list_from_cell_list (src/neighborlist.cpp:496-553) */
static int update_verlet_list_from_cell_list(orc_sys *s) {
  if (nl_reserve(s)) return ORC_E_NOMEM;
  const double ce2 = s->cutoff_extra * s->cutoff_extra;
  const int32_t n = s->n;
  int32_t ind[3];
  for (int32_t i = 0; i < n; ++i) {
    s->nl_start[i] = s->nl.n;
    const double *pi = &s->pos[3 * i];
    binlist_index(s, pi, ind);
    int64_t b = bin_lin(s, ind);
    const int32_t *lst = &s->nbin[b * 27 * 3];
    for (int32_t e = 0; e < s->nbin_n[b]; ++e) {
      int64_t bb = bin_lin(s, &lst[3 * e]);
      for (int32_t k = s->bin_start[bb]; k < s->bin_start[bb] + s->bin_count[bb]; ++k) {
        int32_t j = s->bin_items[k];
        const double *pj;
        if (j >= n) pj = &s->gpos.a[3 * (j - n)];
        else {
          if (j <= i) continue;
          pj = &s->pos[3 * j];
        }
        /* dr = pos[i] - pos[j]; (a-b)^2 == (b-a)^2 bit for bit */
        if (dist2(pi, pj) < ce2 && iv_push(&s->nl, j)) return ORC_E_NOMEM;
      }
    }
    s->nl_count[i] = (int32_t)(s->nl.n - s->nl_start[i]);
  }
  snapshot_old(s);
  return ORC_OK;
}

/* Neighborlist::update_is_needed (src/neighborlist.cpp:100-148) */
static int update_is_needed(orc_sys *s) {
  nl_init(s);
  if (!s->built) return 1;
  const int32_t g = ghost_n(s);
  if (g != s->ghost_old_n) return 1;
  for (int32_t i = 0; i < s->n; ++i)
    if (dist2(&s->pos[3 * i], &s->pos_old_nl[3 * i]) > s->threshold_sq) return 1;
  for (int32_t i = 0; i < g; ++i)
    if (dist2(&s->gpos.a[3 * i], &s->gpos_old_nl.a[3 * i]) > s->threshold_sq) return 1;
  return 0;
}

/* Neighborlist::build (src/neighborlist.cpp:77-98) */
static int nl_build(orc_sys *s, int update) {
  int rc;
  if (s->p.use_cell_list && (rc = update_cell_list(s))) return rc;
  if (!update) update = s->p.rebuild_test ? 1 : update_is_needed(s);
  if (update) {
    if (s->p.use_cell_list) return update_verlet_list_from_cell_list(s);
    return update_verlet_list(s);
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* force_field::Lj::calculate_acceleration (src/force/lj.cpp:393-517)        */
/* ------------------------------------------------------------------------ */
static void lj_acceleration(orc_sys *s) {
  const int32_t nt = s->p.ntypes, n = s->n;
  const double cutoff_sq = s->p.lj_cutoff * s->p.lj_cutoff;
  double c = cutoff_sq;
  double virial = 0.0, pe = 0.0;
  for (int32_t i = 0; i < n; ++i) {
    const double *pi = &s->pos[3 * i];
    const int32_t ti = s->type[i];
    const double minv_i = s->p.mass[ti] == 0.0 ? 0.0 : 1.0 / s->p.mass[ti];
    const int32_t id_i = i;
    for (int64_t k = s->nl_start[i]; k < s->nl_start[i] + s->nl_count[i]; ++k) {
      int32_t j = s->nl.a[k];
      int is_ghost = j >= n;
      const double *pj;
      int32_t tj, id_j;
      if (is_ghost) {
        j -= n;
        pj = &s->gpos.a[3 * j];
        id_j = s->gsrc.a[j];
        tj = s->type[id_j];
      } else {
        pj = &s->pos[3 * j];
        id_j = j;
        tj = s->type[j];
      }
      /* ignore_intra_molecule (:446); a ghost carries its source's molecule index */
      if (s->p.ignore_intra && s->mol[id_i] == s->mol[id_j]) continue;
      const double drx = pj[0] - pi[0], dry = pj[1] - pi[1], drz = pj[2] - pi[2];
      double dr_sq = drx * drx + dry * dry + drz * drz;
      if (s->p.cutoff_list_on) {
        double cl = s->p.cutoff_list[ti * nt + tj];
        c = cl * cl;
      }
      if (dr_sq > c) continue;
      if (dr_sq < s->p.jump_tol) dr_sq = s->p.jump_tol; /* jump_fix (:459-468); jump_tol 0 = off */
      const double eps_ij = s->p.eps[ti * nt + tj];
      if (eps_ij == 0) continue;
      const double sigma_ij = s->p.sigma[ti * nt + tj];
      double r_c_sq_inv = 1 / c;
      double rho_c_sq_inv = sigma_ij * sigma_ij * r_c_sq_inv;
      double rho_c_6_inv = rho_c_sq_inv * rho_c_sq_inv * rho_c_sq_inv;
      double rho_c_12_inv = rho_c_6_inv * rho_c_6_inv;
      double dr_sq_inv = 1 / dr_sq;
      double rho_sq_inv = sigma_ij * sigma_ij * dr_sq_inv;
      double rho_6_inv = rho_sq_inv * rho_sq_inv * rho_sq_inv;
      double rho_12_inv = rho_6_inv * rho_6_inv;
      double forceCoef = 4 * eps_ij *
                         (-12 * rho_12_inv * dr_sq_inv + 6 * rho_6_inv * dr_sq_inv +
                          12 * rho_c_12_inv * r_c_sq_inv - 6 * rho_c_6_inv * r_c_sq_inv);
      if (id_i < id_j) {
        virial += -forceCoef * dr_sq;
        pe += orc_pair_potential(&s->p, ti, tj, dr_sq);
      }
      const double fx = drx * forceCoef, fy = dry * forceCoef, fz = drz * forceCoef;
      s->acc[3 * i] += fx * minv_i;
      s->acc[3 * i + 1] += fy * minv_i;
      s->acc[3 * i + 2] += fz * minv_i;
      if (!is_ghost) {
        const double minv_j = s->p.mass[tj] == 0.0 ? 0.0 : 1.0 / s->p.mass[tj];
        s->acc[3 * j] -= fx * minv_j;
        s->acc[3 * j + 1] -= fy * minv_j;
        s->acc[3 * j + 2] -= fz * minv_j;
      }
    }
  }
  s->virial += virial;
  s->pe = pe;
}

/* Pair potential consistent with the reference force (restated; the
 * reference has none).  With g(r) = U'(r)/r, the reference uses
 * F_i = [g(r) - g(r_c)] (r_j - r_i)  (src/force/lj.cpp:475-484), whose
 * potential is V(r) = U(r) - U(r_c) - 0.5 g(r_c) (r^2 - r_c^2). */
double orc_pair_potential(const orc_params *p, int32_t ti, int32_t tj, double r2) {
  const int32_t nt = p->ntypes;
  double rc = p->cutoff_list_on ? p->cutoff_list[ti * nt + tj] : p->lj_cutoff;
  double c = rc * rc;
  double eps = p->eps[ti * nt + tj], sig = p->sigma[ti * nt + tj];
  if (r2 > c || eps == 0) return 0.0;
  double s2 = sig * sig / r2, s6 = s2 * s2 * s2;
  double sc2 = sig * sig / c, sc6 = sc2 * sc2 * sc2;
  double u = 4 * eps * (s6 * s6 - s6);
  double uc = 4 * eps * (sc6 * sc6 - sc6);
  double gc = 4 * eps * (-12 * sc6 * sc6 / c + 6 * sc6 / c);
  return u - uc - 0.5 * gc * (r2 - c);
}

/* Atom_data::reset_owned_acceleration (src/atom_data.cpp:424-432) */
static void reset_acc(orc_sys *s) { memset(s->acc, 0, (size_t)s->n * 3 * sizeof(double)); }

/* ------------------------------------------------------------------------ */
/* thermo (src/atom_data/kinetic_energy.cpp)                                  */
/* ------------------------------------------------------------------------ */
/* kinetic_energy_mpi_domain (:26-134) for n_r_df 0..3; owned_velocity_cm (:409-453) */
static double kinetic_energy(const orc_sys *s) {
  double e = 0.0;
  const int32_t n = s->n;
  if (s->p.n_r_df == 0) {
    for (int32_t i = 0; i < n; ++i) {
      if (!s->in_domain[i]) continue;
      const double *v = &s->vel[3 * i];
      e += s->p.mass[s->type[i]] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    }
  } else {
    double vc[3] = {0, 0, 0}, msum = 0.0;
    for (int32_t i = 0; i < n; ++i) {
      if (!s->in_domain[i]) continue;
      double m = s->p.mass[s->type[i]];
      msum += m;
      vc[0] += s->vel[3 * i] * m; vc[1] += s->vel[3 * i + 1] * m; vc[2] += s->vel[3 * i + 2] * m;
    }
    vc[0] = vc[0] / msum; vc[1] = vc[1] / msum; vc[2] = vc[2] / msum;
    for (int32_t i = 0; i < n; ++i) {
      if (!s->in_domain[i]) continue;
      double vx = s->vel[3 * i] - vc[0], vy = s->vel[3 * i + 1] - vc[1], vz = s->vel[3 * i + 2] - vc[2];
      e += s->p.mass[s->type[i]] * (vx * vx + vy * vy + vz * vz);
    }
  }
  e *= 0.5;
  return e;
}

/* finalize_temperature_mpi_domain (:189-198), degree_of_freedoms_mpi_domain (:676-715) */
static void finalize_temperature(orc_sys *s) {
  s->ke = kinetic_energy(s);
  int dof = 3 * s->n - s->p.n_r_df;
  s->temperature = 2.0 * s->ke / (s->p.k_b * dof);
}

/* constraint::Nve::apply_thermostat (src/constraint/nve.cpp:132-184) on steps whose
 * index is a multiple of nve_step, then finalize_temperature again */
static void nve_thermostat(orc_sys *s) {
  if (s->p.nve_step <= 0 || s->current_step % s->p.nve_step != 0) return;
  const double energy_now = kinetic_energy(s);
  const double dof = (double)(3 * s->n - s->p.n_r_df); /* degree_of_freedoms() */
  double lambda = 1.0;
  switch (s->p.nve_mode) {
    case 0: lambda = sqrt(s->p.nve_value * dof / energy_now); break;           /* energy_per_dof */
    case 1: lambda = sqrt(s->p.nve_value / energy_now); break;                 /* energy_tot */
    case 2: lambda = sqrt(dof * s->p.nve_value * 0.5 / energy_now); break;     /* kbt */
    default: lambda = sqrt(dof * s->p.nve_kb * s->p.nve_value * 0.5 / energy_now); /* kb, temperature */
  }
  for (int64_t k = 0; k < 3 * (int64_t)s->n; ++k) s->vel[k] *= lambda;
  finalize_temperature(s);
}

/* finalize_pressure_mpi_domain (:238-303) */
static void finalize_pressure(orc_sys *s) {
  if (!s->p.pressure_process) return;
  double volume = s->size_local[0] * s->size_local[1] * s->size_local[2];
  double p2 = (0.0 + 0 + s->virial) / (3.0 * volume);
  double p1 = ((double)s->n * s->p.k_b * s->temperature) / volume;
  s->pressure = p1 + p2;
}

/* ------------------------------------------------------------------------ */
/* Md_simulator (src/md_simulator.cpp)                                        */
/* ------------------------------------------------------------------------ */
/* re_calculate_acc (:422-437) with boundary_condition (:548-563) */
static int re_calculate_acc(orc_sys *s) {
  int upd = exchange_owned(s);
  int rc = exchange_ghost(s);
  if (rc) return rc;
  if ((rc = nl_build(s, upd))) return rc;
  reset_acc(s);
  lj_acceleration(s);
  return ORC_OK;
}

static int any_nan_acc(const orc_sys *s) {
  for (int64_t k = 0; k < 3 * (int64_t)s->n; ++k)
    if (isnan(s->acc[k])) return 1;
  return 0;
}

/* integrate_velocity_verlet (:617-729) */
static int integrate_vv(orc_sys *s) {
  const double dt = s->p.dt;
  const int32_t n = s->n;
  if (any_nan_acc(s)) return ORC_E_NAN;
  for (int32_t i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) {
      double a = s->acc[3 * i + d];
      s->pos[3 * i + d] += s->vel[3 * i + d] * dt + a * 0.5 * dt * dt;
      s->acc_old[3 * i + d] = a;
    }
  int rc = re_calculate_acc(s);
  if (rc) return rc;
  const double hdt = 0.5 * dt;
  for (int32_t i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d)
      s->vel[3 * i + d] += (s->acc[3 * i + d] + s->acc_old[3 * i + d]) * hdt;
  finalize_temperature(s);
  nve_thermostat(s);
  finalize_pressure(s);
  return ORC_OK;
}

/* integrate_leap_frog (:871-980): v += (0.5 dt) a; r += dt v; force; v += (0.5 dt) a */
static int integrate_lf(orc_sys *s) {
  const double dt = s->p.dt, hdt = 0.5 * dt;
  const int32_t n = s->n;
  if (any_nan_acc(s)) return ORC_E_NAN;
  for (int32_t i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) {
      s->vel[3 * i + d] += hdt * s->acc[3 * i + d];
      s->pos[3 * i + d] += dt * s->vel[3 * i + d];
    }
  int rc = re_calculate_acc(s);
  if (rc) return rc;
  for (int32_t i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) s->vel[3 * i + d] += hdt * s->acc[3 * i + d];
  finalize_temperature(s);
  nve_thermostat(s);
  finalize_pressure(s);
  return ORC_OK;
}

/* integrate_velocity_verlet_langevin (:731-869) and its coefficients (:394-416) */
static int integrate_langevin(orc_sys *s) {
  const double dt = s->p.dt;
  const double fr = s->p.lang_friction;
  const double la = (2.0 - fr * dt) / (2.0 + fr * dt);
  double lb;
  if (s->p.lang_kbt > 0) lb = sqrt(s->p.lang_kbt * fr * 0.5 * dt);
  else if (s->p.lang_kb > 0 && s->p.lang_temperature > 0)
    lb = sqrt(s->p.lang_kb * s->p.lang_temperature * fr * 0.5 * dt);
  else return ORC_E_ARG;
  const double lc = 2.0 * dt / (2.0 + fr * dt);
  const int32_t n = s->n;
  double *eta = (double *)malloc((size_t)n * 3 * sizeof(double));
  if (!eta) return ORC_E_NOMEM;
  for (int32_t i = 0; i < n; ++i) {
    if (s->p.noise_mode == 1) orc_langevin_eta(s->p.seed, (uint64_t)s->current_step, (uint32_t)i, &eta[3 * i]);
    else eta[3 * i] = eta[3 * i + 1] = eta[3 * i + 2] = 0.0;
  }
  if (any_nan_acc(s)) { free(eta); return ORC_E_NAN; }
  for (int32_t i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d)
      s->vel[3 * i + d] += s->acc[3 * i + d] * 0.5 * dt + eta[3 * i + d] * lb;
  finalize_temperature(s);
  nve_thermostat(s); /* constraints' apply_thermostat on the mid-step velocities (:784-791) */
  finalize_pressure(s);
  for (int32_t i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) s->pos[3 * i + d] += s->vel[3 * i + d] * lc;
  int rc = re_calculate_acc(s);
  if (rc) { free(eta); return rc; }
  for (int32_t i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d)
      s->vel[3 * i + d] = s->vel[3 * i + d] * la + eta[3 * i + d] * lb + s->acc[3 * i + d] * 0.5 * dt;
  free(eta);
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* public entry points                                                        */
/* ------------------------------------------------------------------------ */
orc_sys *orc_new(const orc_params *p, int32_t n, const double *pos3, const double *vel3, const int32_t *type) {
  if (!p || n < 0 || p->ntypes < 1 || p->ntypes > ORC_MAX_TYPES) return NULL;
  orc_sys *s = (orc_sys *)calloc(1, sizeof(orc_sys));
  if (!s) return NULL;
  s->p = *p;
  s->n = n;
  size_t b3 = ((size_t)n + 1) * 3 * sizeof(double);
  s->pos = (double *)malloc(b3); s->vel = (double *)malloc(b3);
  s->acc = (double *)calloc(1, b3); s->acc_old = (double *)calloc(1, b3);
  s->pos_old_nl = (double *)calloc(1, b3);
  s->type = (int32_t *)malloc(((size_t)n + 1) * sizeof(int32_t));
  s->in_domain = (unsigned char *)calloc((size_t)n + 1, 1);
  s->img = (int32_t *)calloc(((size_t)n + 1) * 3, sizeof(int32_t));
  s->mol = (int32_t *)malloc(((size_t)n + 1) * sizeof(int32_t));
  if (s->mol) for (int32_t i = 0; i < n; ++i) s->mol[i] = -1;  /* Atom_data::add_atom (src/atom_data.cpp:625) */
  if (!s->mol || !s->img || !s->in_domain || !s->pos || !s->vel || !s->acc || !s->acc_old || !s->pos_old_nl || !s->type) { orc_free(s); return NULL; }
  memcpy(s->pos, pos3, (size_t)n * 3 * sizeof(double));
  memcpy(s->vel, vel3, (size_t)n * 3 * sizeof(double));
  memcpy(s->type, type, (size_t)n * sizeof(int32_t));
  for (int d = 0; d < 3; ++d) {
    s->size[d] = p->hi[d] - p->lo[d];
    /* calculate_local_domain with grid_index 0 of 1 */
    s->lo_local[d] = p->lo[d] + (p->hi[d] - p->lo[d]) * 0 / 1;
    s->hi_local[d] = p->lo[d] + (p->hi[d] - p->lo[d]) * 1 / 1;
    s->size_local[d] = s->hi_local[d] - s->lo_local[d];
  }
  return s;
}

void orc_free(orc_sys *s) {
  if (!s) return;
  free(s->pos); free(s->vel); free(s->acc); free(s->acc_old); free(s->pos_old_nl); free(s->type); free(s->in_domain);
  free(s->img); free(s->mol);
  free(s->gpos.a); free(s->gsrc.a); free(s->gshift.a); free(s->gpos_old_nl.a);
  free(s->bin_start); free(s->bin_count); free(s->bin_items); free(s->nbin_n); free(s->nbin);
  free(s->nl_start); free(s->nl_count); free(s->nl.a);
  free(s);
}

/* Atom_data::set_atoms_mpi_rank (src/atom_data.cpp:817-839) with
 * position_inside_local_domain (:516-546): atoms outside [lo, hi) at
 * initialisation are foreign for the rest of the run, which removes them from
 * the kinetic energy (src/atom_data/kinetic_energy.cpp:41, 427). */
static void set_atoms_mpi_rank(orc_sys *s) {
  for (int32_t i = 0; i < s->n; ++i) {
    const double *q = &s->pos[3 * i];
    int in = 1;
    for (int d = 0; d < 3; ++d)
      if (q[d] < s->lo_local[d] || q[d] >= s->hi_local[d]) in = 0;
    s->in_domain[i] = (unsigned char)in;
  }
}

/* Md_simulator::setup (:565-611) after initialize (:366-420) */
int32_t orc_setup(orc_sys *s) {
  set_atoms_mpi_rank(s);
  int rc = nl_init(s);
  if (rc) return rc;
  exchange_owned(s);
  if ((rc = exchange_ghost(s))) return rc;
  if ((rc = nl_build(s, 1))) return rc;
  reset_acc(s);
  s->virial = 0.0;
  lj_acceleration(s);
  finalize_temperature(s);
  s->setup_done = 1;
  return ORC_OK;
}

/* Md_simulator::step (:445-546) */
int32_t orc_step(orc_sys *s, int32_t nsteps) {
  if (!s->setup_done) {
    int rc = orc_setup(s);
    if (rc) return rc;
  }
  for (int32_t k = 0; k < nsteps; ++k) {
    s->virial = 0.0;
    int rc = s->p.integrator == 1 ? integrate_langevin(s) : (s->p.integrator == 2 ? integrate_lf(s) : integrate_vv(s));
    if (rc) return rc;
    s->current_step++;
  }
  return ORC_OK;
}

int32_t orc_set_molecules(orc_sys *s, const int32_t *mol) {
  if (!s || !mol) return ORC_E_ARG;
  memcpy(s->mol, mol, (size_t)s->n * sizeof(int32_t));
  return ORC_OK;
}

void orc_get_images(const orc_sys *s, int32_t *img3) {
  memcpy(img3, s->img, (size_t)s->n * 3 * sizeof(int32_t));
}

void orc_get_state(const orc_sys *s, double *pos3, double *vel3, double *acc3) {
  size_t b = (size_t)s->n * 3 * sizeof(double);
  if (pos3) memcpy(pos3, s->pos, b);
  if (vel3) memcpy(vel3, s->vel, b);
  if (acc3) memcpy(acc3, s->acc, b);
}

/* o[0] is Atom_data::kinetic_energy() of the current velocities: for Langevin the
 * temperature was taken mid-step, the kinetic energy is read after it */
void orc_get_thermo(const orc_sys *s, double *o) {
  o[0] = kinetic_energy(s); o[1] = s->temperature; o[2] = s->pressure; o[3] = s->virial; o[4] = s->pe;
  o[5] = (double)s->rebuilds;
}

int64_t orc_current_step(const orc_sys *s) { return s->current_step; }

int64_t orc_pair_count(const orc_sys *s) {
  int64_t c = 0;
  for (int32_t i = 0; i < s->n; ++i)
    for (int64_t k = s->nl_start[i]; k < s->nl_start[i] + s->nl_count[i]; ++k)
      c += s->nl.a[k] >= s->n ? 1 : 2;
  return c;
}

int64_t orc_get_pairs(const orc_sys *s, int32_t *o, int64_t cap) {
  int64_t c = 0;
  for (int32_t i = 0; i < s->n; ++i)
    for (int64_t k = s->nl_start[i]; k < s->nl_start[i] + s->nl_count[i]; ++k) {
      int32_t j = s->nl.a[k];
      if (j >= s->n) {
        int32_t g = j - s->n;
        if (c < cap) {
          int32_t *r = &o[5 * c];
          r[0] = i; r[1] = s->gsrc.a[g];
          r[2] = s->gshift.a[3 * g]; r[3] = s->gshift.a[3 * g + 1]; r[4] = s->gshift.a[3 * g + 2];
        }
        ++c;
      } else {
        if (c + 1 < cap) {
          int32_t *r = &o[5 * c];
          r[0] = i; r[1] = j; r[2] = r[3] = r[4] = 0;
          r[5] = j; r[6] = i; r[7] = r[8] = r[9] = 0;
        }
        c += 2;
      }
    }
  return c;
}

int32_t orc_ghost_count(const orc_sys *s) { return ghost_n(s); }

void orc_get_ghosts(const orc_sys *s, int32_t *src, int32_t *shift3, double *pos3) {
  int32_t g = ghost_n(s);
  if (src) memcpy(src, s->gsrc.a, (size_t)g * sizeof(int32_t));
  if (shift3) memcpy(shift3, s->gshift.a, (size_t)g * 3 * sizeof(int32_t));
  if (pos3) memcpy(pos3, s->gpos.a, (size_t)g * 3 * sizeof(double));
}

void orc_get_bins(const orc_sys *s, int32_t *owned3, int32_t *ghost3) {
  int32_t ind[3];
  if (owned3)
    for (int32_t i = 0; i < s->n; ++i) {
      binlist_index(s, &s->pos[3 * i], ind);
      owned3[3 * i] = ind[0]; owned3[3 * i + 1] = ind[1]; owned3[3 * i + 2] = ind[2];
    }
  if (ghost3)
    for (int32_t g = 0; g < ghost_n(s); ++g) {
      binlist_index(s, &s->gpos.a[3 * g], ind);
      ghost3[3 * g] = ind[0]; ghost3[3 * g + 1] = ind[1]; ghost3[3 * g + 2] = ind[2];
    }
}

void orc_get_nbins(const orc_sys *s, int32_t *nb3) { nb3[0] = s->nb[0]; nb3[1] = s->nb[1]; nb3[2] = s->nb[2]; }
