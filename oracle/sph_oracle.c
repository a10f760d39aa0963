/*
 * sph_oracle.c -- CPU oracle (test infrastructure only; see sph_oracle.h).
 *
 * Every function below names the reference lines it restates.  Arithmetic is
 * IEEE double with no contraction (built with -ffp-contract=off, no fast-math)
 * so that each expression rounds exactly where it is written.  The parallel
 * loops split the OUTER loop over target particles only: each target's own
 * summation order is the reference's, so results do not depend on the number
 * of threads, exactly as in the reference (core.jl:126 threads over p).
 *
 * Evaluation order shared with the GPU library (the definition of the FP64
 * path; kernels.jl is @fastmath, so this is one admissible reading of it):
 *   r   = sqrt(fma(d2, d2, fma(d1, d1, d0 * d0)))   the kernel distance (the
 *         support test keeps the reference's unfused dist, core.jl:8-10)
 *   t   = fma(-r, 1/H, 1) (= 1 - x, x = r/H; 1/H computed once), 0 when < 0
 *   W   = (Cw * (t2 * t2)) * fma(-4, t, 5),  t2 = t*t  (5 - 4t = 1 + 4x)
 *         Cw = 7/pi / H^2 (2D), 21/(2 pi) / H^3 (3D), H^2 = H*H, H^3 = H^2*H
 *   rDW = Cr * (t2 * t)
 *         Cr = -140/pi / H^4 (2D), -210/pi / H^5 (3D), H^4 = H^2*H^2, H^5 = H^4*H
 *   the mass is folded into the constants (m Cw, m Cr) in the pair operators
 */
#include "sph_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

struct orc_system {
  orc_params p;
  int kdim;                 /* kernel dimension (params.dim)             */
  int64_t key_phase[3], key_lim[3], key_max;
  int64_t key_diff[27];
  int n_diff;
  /* derived constants, computed once */
  double inv_h, cw, cr, B, hdt, eta2, alpha_c0, gmag;
  double mcw, mcr, ca; /* m C_w, m C_r, -(alpha c0) h_smooth */
  double mcw5, mcw4;   /* 5 m C_w and -4 m C_w: m W = t^4 (5 m C_w - 4 m C_w t) */
  double c2, rho0sq;   /* c0^2, rho0^2 (ORC_EOS_LINEAR) */
  /* particles in the reference's order (0-based index = position in
   * sys.particles minus one) */
  int64_t n, cap;
  double (*x)[3], (*v)[3], (*a)[3], (*xs)[3];
  double *rho, *rho_ref, *P, *Pr;
  int32_t* type;
  int64_t* oid;
  int64_t next_oid;
  /* cell lists (CSR): cell k (1-based) holds entries[cstart[k] .. cstart[k+1]) */
  int64_t* cstart;
  int64_t* entries;
  int64_t* keys;
  int cells_valid;
};

/* ---------------------------------------------------------------- kernels */
/* The Wendland quintic (kernels.jl:108-115 wendland2, :156-163 wendland3)
 * and its derivative over r (kernels.jl:140-147, :188-195) are @fastmath in
 * the reference; both implementations evaluate them in this one order:
 * t = 1 - r (1/h) as one fused operation, 0 beyond the support,
 * W = (C_w t^4)(5 - 4t) (5 - 4t = 1 + 4x), rDW = C_r t^3. */
static inline double ker_t(const orc_system* s, double r) {
  const double t = fma(-r, s->inv_h, 1.0);
  return t < 0.0 ? 0.0 : t;
}
static inline double ker_w(const orc_system* s, double r) {
  const double t = ker_t(s, r);
  const double t2 = t * t;
  return (s->cw * (t2 * t2)) * fma(-4.0, t, 5.0);
}
static inline double ker_rdw(const orc_system* s, double r) {
  const double t = ker_t(s, r);
  return s->cr * ((t * t) * t);
}
/* the distance a kernel is evaluated at: sqrt((d0 d0 + d1 d1) + d2 d2) with
 * the sum fused (the support test keeps the reference's unfused dist) */
static inline double ker_r(const double d[3]) {
  return sqrt(fma(d[2], d[2], fma(d[1], d[1], d[0] * d[0])));
}

/* ------------------------------------------------------------ construction */
/* structs.jl:57-92 */
orc_system* orc_create(const orc_params* p) {
  if (!(p->h > 0.0)) return NULL; /* structs.jl:59 */
  if (p->eos != ORC_EOS_TAIT && p->eos != ORC_EOS_LINEAR) return NULL;
  orc_system* s = (orc_system*)calloc(1, sizeof(orc_system));
  s->p = *p;
  s->kdim = p->dim;
  for (int d = 0; d < 3; ++d) {
    s->key_phase[d] = (int64_t)floor(p->domain_min[d] / p->h);                      /* :66 */
    s->key_lim[d] = (int64_t)floor(p->domain_max[d] / p->h) - s->key_phase[d] + 1;  /* :67 */
  }
  s->key_max = s->key_lim[0] * s->key_lim[1] * s->key_lim[2]; /* :68 */
  s->n_diff = 0;
  if (s->key_lim[2] == 1) { /* :73-75, di outer, dj inner */
    for (int di = -1; di <= 1; ++di)
      for (int dj = -1; dj <= 1; ++dj) s->key_diff[s->n_diff++] = di + s->key_lim[0] * dj;
  } else { /* :79-81, di outer, dj middle, dk inner */
    for (int di = -1; di <= 1; ++di)
      for (int dj = -1; dj <= 1; ++dj)
        for (int dk = -1; dk <= 1; ++dk)
          s->key_diff[s->n_diff++] = di + s->key_lim[0] * (dj + s->key_lim[1] * dk);
  }
  const double H = p->h;
  s->inv_h = 1.0 / H;
  const double h2 = H * H;
  if (s->kdim == 2) {
    s->cw = 2.228169203286535 / h2;
    s->cr = -44.563384065730695 / (h2 * h2);
  } else {
    s->cw = 3.3422538049298023 / (h2 * H);
    s->cr = -66.84507609859604 / ((h2 * h2) * H);
  }
  s->B = ((p->c0 * p->c0) * p->rho0) / 7.0;
  s->c2 = p->c0 * p->c0;          /* test_collision_2d.jl:72 c^2 */
  s->rho0sq = p->rho0 * p->rho0;  /* test_collision_2d.jl:77 rho0^2 */
  s->hdt = 0.5 * p->dt;
  s->eta2 = 0.01 * (p->h_smooth * p->h_smooth);
  s->alpha_c0 = p->alpha * p->c0;
  s->mcw = p->mass * s->cw;
  s->mcw5 = 5.0 * s->mcw;
  s->mcw4 = -4.0 * s->mcw;
  s->mcr = p->mass * s->cr;
  s->ca = -(s->alpha_c0 * p->h_smooth);
  s->gmag = fabs(p->gravity[p->vertical_axis]);
  s->cstart = (int64_t*)calloc((size_t)(s->key_max + 2), sizeof(int64_t));
  return s;
}

void orc_destroy(orc_system* s) {
  if (!s) return;
  free(s->x); free(s->v); free(s->a); free(s->xs);
  free(s->rho); free(s->rho_ref); free(s->P); free(s->Pr);
  free(s->type); free(s->oid); free(s->cstart); free(s->entries); free(s->keys);
  free(s);
}

int orc_dim(const orc_system* s) { return s->key_lim[2] == 1 ? 2 : 3; }

void orc_geometry(const orc_system* s, int64_t key_phase[3], int64_t key_lim[3],
                  int64_t* key_max, int64_t key_diff[27], int32_t* n_diff) {
  for (int d = 0; d < 3; ++d) { key_phase[d] = s->key_phase[d]; key_lim[d] = s->key_lim[d]; }
  *key_max = s->key_max;
  for (int i = 0; i < s->n_diff; ++i) key_diff[i] = s->key_diff[i];
  *n_diff = s->n_diff;
}

static void reserve(orc_system* s, int64_t cap) {
  if (cap <= s->cap) return;
  size_t c = (size_t)cap;
  s->x = realloc(s->x, c * sizeof(*s->x));
  s->v = realloc(s->v, c * sizeof(*s->v));
  s->a = realloc(s->a, c * sizeof(*s->a));
  s->xs = realloc(s->xs, c * sizeof(*s->xs));
  s->rho = realloc(s->rho, c * sizeof(double));
  s->rho_ref = realloc(s->rho_ref, c * sizeof(double));
  s->P = realloc(s->P, c * sizeof(double));
  s->Pr = realloc(s->Pr, c * sizeof(double));
  s->type = realloc(s->type, c * sizeof(int32_t));
  s->oid = realloc(s->oid, c * sizeof(int64_t));
  s->entries = realloc(s->entries, c * sizeof(int64_t));
  s->keys = realloc(s->keys, c * sizeof(int64_t));
  s->cap = cap;
}

/* grids.jl:253-258 generate_particles! (push! in order) */
int orc_add_particles(orc_system* s, int64_t n, const double* x, const double* v,
                      const double* rho, const double* rho_ref, const int32_t* type) {
  reserve(s, s->n + n);
  for (int64_t i = 0; i < n; ++i) {
    int64_t j = s->n + i;
    for (int d = 0; d < 3; ++d) {
      s->x[j][d] = x[3 * i + d];
      s->v[j][d] = v ? v[3 * i + d] : 0.0;
      s->a[j][d] = 0.0;
      s->xs[j][d] = 0.0;
    }
    s->rho[j] = rho ? rho[i] : 0.0;
    s->rho_ref[j] = rho_ref ? rho_ref[i] : 0.0;
    s->P[j] = 0.0;
    s->Pr[j] = 0.0;
    s->type[j] = type ? type[i] : ORC_FLUID;
    s->oid[j] = s->next_oid++;
  }
  s->n += n;
  s->cells_valid = 0;
  return 0;
}

int64_t orc_num_particles(const orc_system* s) { return s->n; }

void orc_get_state(const orc_system* s, double* x, double* v, double* a, double* xsph,
                   double* rho, double* rho_ref, double* P, int32_t* type, int64_t* oid) {
  for (int64_t i = 0; i < s->n; ++i) {
    for (int d = 0; d < 3; ++d) {
      if (x) x[3 * i + d] = s->x[i][d];
      if (v) v[3 * i + d] = s->v[i][d];
      if (a) a[3 * i + d] = s->a[i][d];
      if (xsph) xsph[3 * i + d] = s->xs[i][d];
    }
    if (rho) rho[i] = s->rho[i];
    if (rho_ref) rho_ref[i] = s->rho_ref[i];
    if (P) P[i] = s->P[i];
    if (type) type[i] = s->type[i];
    if (oid) oid[i] = s->oid[i];
  }
}

void orc_set_state(orc_system* s, const double* x, const double* v, const double* a,
                   const double* xsph, const double* rho, const double* rho_ref,
                   const double* P) {
  for (int64_t i = 0; i < s->n; ++i) {
    for (int d = 0; d < 3; ++d) {
      if (x) s->x[i][d] = x[3 * i + d];
      if (v) s->v[i][d] = v[3 * i + d];
      if (a) s->a[i][d] = a[3 * i + d];
      if (xsph) s->xs[i][d] = xsph[3 * i + d];
    }
    if (rho) s->rho[i] = rho[i];
    if (rho_ref) s->rho_ref[i] = rho_ref[i];
    if (P) {
      s->P[i] = P[i];
      s->Pr[i] = s->type[i] != ORC_FLUID      ? 0.0
                 : s->p.eos == ORC_EOS_LINEAR ? P[i] / s->rho0sq
                                              : P[i] / (s->rho[i] * s->rho[i]);
    }
  }
  if (x) s->cells_valid = 0;
}

/* ---------------------------------------------------------------- binning */
/* structs.jl:97-106.  Int64(floor(..)) throws for NaN, Inf and values outside
 * the Int64 range; the reference catches that and returns -1. */
int64_t orc_find_key(const orc_system* s, const double x[3]) {
  int64_t ijk[3];
  for (int d = 0; d < 3; ++d) {
    double f = floor(x[d] / s->p.h);
    if (!(f >= -9223372036854775808.0 && f < 9223372036854775808.0)) return -1;
    ijk[d] = 1 + (int64_t)f - s->key_phase[d];
  }
  return ijk[0] + s->key_lim[0] * (ijk[1] - 1) + s->key_lim[0] * s->key_lim[1] * (ijk[2] - 1);
}

/* geometry.jl:24-30 is_inside(x, ::Box); comparisons are false for NaN */
static inline int inside_box(const orc_system* s, const double x[3]) {
  for (int d = 0; d < 3; ++d)
    if (!(s->p.domain_min[d] <= x[d] && x[d] <= s->p.domain_max[d])) return 0;
  return 1;
}

static void copy_particle(orc_system* s, int64_t dst, int64_t src) {
  if (dst == src) return;
  for (int d = 0; d < 3; ++d) {
    s->x[dst][d] = s->x[src][d];
    s->v[dst][d] = s->v[src][d];
    s->a[dst][d] = s->a[src][d];
    s->xs[dst][d] = s->xs[src][d];
  }
  s->rho[dst] = s->rho[src];
  s->rho_ref[dst] = s->rho_ref[src];
  s->P[dst] = s->P[src];
  s->Pr[dst] = s->Pr[src];
  s->type[dst] = s->type[src];
  s->oid[dst] = s->oid[src];
}

/* core.jl:51-90 */
void orc_create_cell_list(orc_system* s) {
  const int64_t n = s->n;
  /* core.jl:63-69: removal cell collects indices outside the bounding box;
   * add_index! keeps them in descending order (core.jl:26-41). */
  int64_t k = 0;
  int64_t* rem = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i)
    if (!inside_box(s, s->x[i])) rem[k++] = i; /* ascending here */
  /* core.jl:71-81: particles[removal[i]] = particles[end+1-i] for the removal
   * entries in descending order, then resize! */
  for (int64_t t = 0; t < k; ++t) copy_particle(s, rem[k - 1 - t], n - 1 - t);
  free(rem);
  s->n = n - k;
  /* core.jl:83-89: every cell holds its particle indices in descending order
   * (add_index! bubbles each insertion into place, core.jl:31-37). */
  const int64_t m = s->n;
  memset(s->cstart, 0, (size_t)(s->key_max + 2) * sizeof(int64_t));
  for (int64_t i = 0; i < m; ++i) {
    int64_t key = orc_find_key(s, s->x[i]);
    s->keys[i] = key;
    if (key < 1 || key > s->key_max) abort(); /* cannot happen inside the box */
    s->cstart[key + 1] += 1;
  }
  for (int64_t c = 1; c <= s->key_max; ++c) s->cstart[c + 1] += s->cstart[c];
  int64_t* fill = (int64_t*)malloc((size_t)(s->key_max + 2) * sizeof(int64_t));
  memcpy(fill, s->cstart, (size_t)(s->key_max + 2) * sizeof(int64_t));
  for (int64_t i = m - 1; i >= 0; --i) s->entries[fill[s->keys[i]]++] = i;
  free(fill);
  s->cells_valid = 1;
}

void orc_keys(const orc_system* s, int64_t* keys) {
  for (int64_t i = 0; i < s->n; ++i) keys[i] = s->keys[i];
}

/* -------------------------------------------------------------- pair loop */
/* core.jl:8-10 + algebra.jl:49-60: r = sqrt((d1*d1 + d2*d2) + d3*d3) */
static inline double dist2(const double* xp, const double* xq, double d[3]) {
  d[0] = xp[0] - xq[0];
  d[1] = xp[1] - xq[1];
  d[2] = xp[2] - xq[2];
  return (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
}

/* core.jl:94-112 for one target p and one built-in operator.  Operator bodies:
 *   density      find_rho! (collapse_symplectic.jl:98-102), fluid targets,
 *                every neighbour (walls take part in the sum)
 *   force        internal_force! (collapse_symplectic.jl:114-118) with the
 *                Tait pressure, plus Monaghan viscosity and XSPH between fluid
 *                particles; wall neighbours contribute the pressure term with
 *                the wall pressure of the wall-pressure pass
 *   wall pressure  wall targets: P_w = (sum_f P_f W + sum_f rho_f (g . x_wf) W)
 *                / sum_f W over fluid neighbours (Adami, Hu & Adams 2012) */
static int64_t binary_one(orc_system* s, int op, int64_t p) {
  const double H = s->p.h;
  const int64_t key = orc_find_key(s, s->x[p]); /* core.jl:95 */
  const int tp = s->type[p];
  const int active = op == ORC_OP_WALL_PRESSURE ? tp == ORC_WALL : tp == ORC_FLUID;
  if (!active) return 0; /* the operator does nothing for this target */
  const double* xp = s->x[p];
  const double* g = s->p.gravity;
  int64_t pairs = 0;
  double acc = op == ORC_OP_DENSITY ? s->rho[p] : s->rho_ref[p];
  double ax = s->a[p][0], ay = s->a[p][1], az = s->a[p][2];
  double sx = s->xs[p][0], sy = s->xs[p][1], sz = s->xs[p][2];
  /* XSPH: sum_q wx (v_q - v_p) formed as sum_q wx v_q - v_p sum_q wx, the
   * two sums in the neighbour order */
  double xw = 0.0, xv0 = 0.0, xv1 = 0.0, xv2 = 0.0;
  double wp = 0.0, wg = 0.0, ws = 0.0;
  const double* vp = s->v[p];
  const double rhop = s->rho[p], prp = s->Pr[p];
  for (int c = 0; c < s->n_diff; ++c) { /* core.jl:96 */
    const int64_t nk = key + s->key_diff[c];
    if (!(1 <= nk && nk <= s->key_max)) continue; /* core.jl:98 */
    for (int64_t e = s->cstart[nk]; e < s->cstart[nk + 1]; ++e) {
      const int64_t q = s->entries[e];
      double d[3];
      const double r = sqrt(dist2(xp, s->x[q], d));
      if (r > H || p == q) continue; /* core.jl:105 */
      const int tq = s->type[q];
      /* pairs the operator acts on: every neighbour, except that the wall
       * pressure only sums fluid neighbours */
      if (op != ORC_OP_WALL_PRESSURE || tq == ORC_FLUID) ++pairs;
      /* the kernel pieces on a hit (ker_w / ker_rdw above) at the kernel
       * distance, with the particle mass folded into the constants; the
       * density adds m W rounded (a per-pair value), the other sums are
       * formed with fused multiply-adds */
      const double rk = ker_r(d);
      const double t = ker_t(s, rk);
      const double t2 = t * t;
      if (op == ORC_OP_DENSITY || op == ORC_OP_DENSITY_REF) {
        acc = acc + (t2 * t2) * fma(s->mcw4, t, s->mcw5); /* + m W */
      } else if (op == ORC_OP_WALL_PRESSURE) {
        if (tq == ORC_FLUID) {
          const double w = (s->cw * (t2 * t2)) * fma(-4.0, t, 5.0);
          const double gd = fma(g[2], d[2], fma(g[1], d[1], g[0] * d[0]));
          wp = fma(s->P[q], w, wp);
          wg = fma(s->rho[q] * gd, w, wg);
          ws = ws + w;
        }
      } else if (tq == ORC_FLUID) {
        const double ker = s->mcr * (t2 * t); /* m rDW */
        const double dv0 = vp[0] - s->v[q][0], dv1 = vp[1] - s->v[q][1], dv2 = vp[2] - s->v[q][2];
        const double vdx = fma(dv2, d[2], fma(dv1, d[1], dv0 * d[0]));
        const double inv_rb = 2.0 / (rhop + s->rho[q]);
        double pi = 0.0;
        if (vdx < 0.0) {
          /* Monaghan: -alpha c0 mu / rho_bar, mu = h v.x / (r^2 + eta^2),
           * r^2 + eta^2 as one fused multiply-add, the quotient as a product
           * with the reciprocal */
          pi = ((s->ca * vdx) * (1.0 / fma(rk, rk, s->eta2))) * inv_rb;
        }
        const double cf = -ker * ((prp + s->Pr[q]) + pi);
        ax = fma(cf, d[0], ax);
        ay = fma(cf, d[1], ay);
        az = fma(cf, d[2], az);
        const double wx = ((t2 * t2) * fma(s->mcw4, t, s->mcw5)) * inv_rb; /* m W / rho_bar */
        xw = xw + wx;
        xv0 = fma(wx, s->v[q][0], xv0);
        xv1 = fma(wx, s->v[q][1], xv1);
        xv2 = fma(wx, s->v[q][2], xv2);
      } else {
        /* wall neighbour: pressure term only */
        const double ker = s->mcr * (t2 * t);
        const double cf = -ker * (prp + s->Pr[q]);
        ax = fma(cf, d[0], ax);
        ay = fma(cf, d[1], ay);
        az = fma(cf, d[2], az);
      }
    }
  }
  if (op == ORC_OP_DENSITY) s->rho[p] = acc;
  else if (op == ORC_OP_DENSITY_REF) s->rho_ref[p] = acc;
  else if (op == ORC_OP_WALL_PRESSURE) {
    const double P = ws > 0.0 ? (wp + wg) / ws : 0.0;
    s->P[p] = P;
    s->Pr[p] = P / (s->p.rho0 * s->p.rho0);
    s->rho[p] = s->p.rho0;
  } else {
    s->a[p][0] = ax; s->a[p][1] = ay; s->a[p][2] = az;
    s->xs[p][0] = sx + fma(-vp[0], xw, xv0);
    s->xs[p][1] = sy + fma(-vp[1], xw, xv1);
    s->xs[p][2] = sz + fma(-vp[2], xw, xv2);
  }
  return pairs;
}

/* op!(p, p, 0.0) for the self term (core.jl:155-157) */
static void self_one(orc_system* s, int op, int64_t p) {
  if (s->type[p] != ORC_FLUID || op == ORC_OP_WALL_PRESSURE) return;
  const double m = s->p.mass;
  if (op == ORC_OP_DENSITY) s->rho[p] = s->rho[p] + m * ker_w(s, 0.0);
  else if (op == ORC_OP_DENSITY_REF) s->rho_ref[p] = s->rho_ref[p] + m * ker_w(s, 0.0);
  else {
    /* force with q == p, r == 0: every term is a product with a zero vector */
    const double ker = m * ker_rdw(s, 0.0);
    const double inv_rb = 2.0 / (s->rho[p] + s->rho[p]);
    const double cf = -ker * ((s->Pr[p] + s->Pr[p]) + 0.0);
    const double wx = (m * ker_w(s, 0.0)) * inv_rb;
    for (int d = 0; d < 3; ++d) {
      s->a[p][d] = s->a[p][d] + cf * 0.0;
      s->xs[p][d] = s->xs[p][d] + wx * (s->v[p][d] - s->v[p][d]);
    }
  }
}

/* core.jl:125-129 apply_binary! and core.jl:151-161 apply! */
int64_t orc_apply(orc_system* s, int op, int self) {
  /* positions moved since create_cell_list!: the reference would traverse
   * stale cells (core.jl:44-49 docstring); refuse instead */
  if (!s->cells_valid) return -1;
  int64_t pairs = 0;
  const int64_t n = s->n;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : pairs)
  for (int64_t p = 0; p < n; ++p) pairs += binary_one(s, op, p);
  if (self) {
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) self_one(s, op, p);
  }
  return pairs;
}

/* core.jl:138-142 apply_unary! with the built-in unary operators */
void orc_apply_unary(orc_system* s, int op) {
  const int64_t n = s->n;
  const orc_params* P = &s->p;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const int fluid = s->type[i] == ORC_FLUID;
    switch (op) {
      case ORC_OP_RESET_RHO: s->rho[i] = 0.0; break;
      case ORC_OP_RESET_RHO_REF: s->rho_ref[i] = 0.0; break;
      case ORC_OP_RESET_A:
        for (int d = 0; d < 3; ++d) { s->a[i][d] = 0.0; s->xs[i][d] = 0.0; }
        break;
      case ORC_OP_EOS:
        if (fluid && P->eos == ORC_EOS_LINEAR) {
          /* test_collision_2d.jl:71-73 find_pressure!: P = c^2 (rho - rho0);
           * :77 uses P / rho0^2 */
          s->P[i] = s->c2 * (s->rho[i] - s->rho_ref[i]);
          s->Pr[i] = s->P[i] / s->rho0sq;
        } else if (fluid) {
          const double ratio = s->rho[i] / s->rho_ref[i];
          const double r2 = ratio * ratio;
          const double r4 = r2 * r2;
          const double r7 = (r4 * r2) * ratio;
          s->P[i] = s->B * (r7 - 1.0);
          s->Pr[i] = s->P[i] / (s->rho[i] * s->rho[i]);
        } else {
          s->P[i] = 0.0;
          s->Pr[i] = 0.0;
        }
        break;
      case ORC_OP_KICK: /* collapse_symplectic.jl:139-143 accelerate! */
        if (fluid)
          for (int d = 0; d < 3; ++d) s->v[i][d] = s->v[i][d] + s->hdt * (s->a[i][d] + P->gravity[d]);
        break;
      case ORC_OP_DRIFT: /* collapse_symplectic.jl:133-137 move! */
        if (fluid)
          for (int d = 0; d < 3; ++d)
            s->x[i][d] = s->x[i][d] + P->dt * (s->v[i][d] + P->eps_xsph * s->xs[i][d]);
        break;
      case ORC_OP_HYDROSTATIC:
        if (fluid) {
          const double y = s->x[i][P->vertical_axis];
          const double u = (P->rho0 * s->gmag * (P->col_height - y)) / s->B;
          const double c = 1.0 + u;
          double f = 1.0 + u / 7.0;
          for (int it = 0; it < 6; ++it) { /* Newton for f^7 = c */
            const double f2 = f * f;
            const double f3 = f2 * f;
            const double f6 = f3 * f3;
            const double f7 = f6 * f;
            f = f - (f7 - c) / (7.0 * f6);
          }
          s->rho_ref[i] = s->rho_ref[i] / f;
        }
        break;
      default: break;
    }
  }
  if (op == ORC_OP_DRIFT) s->cells_valid = 0;
}

/* ------------------------------------------------------------------- sums */
static inline double sum_func(const orc_system* s, int func, int64_t q, double r) {
  const double m = s->p.mass;
  const int tq = s->type[q];
  switch (func) {
    case ORC_SUM_DENSITY: return m * ker_w(s, r);
    case ORC_SUM_KERNEL: return ker_w(s, r);
    case ORC_SUM_PRESSURE: return tq == ORC_FLUID ? ((m / s->rho[q]) * s->P[q]) * ker_w(s, r) : 0.0;
    case ORC_SUM_SHEPARD: return tq == ORC_FLUID ? (m / s->rho[q]) * ker_w(s, r) : 0.0;
    default: return 0.0;
  }
}

/* core.jl:240-260 (point) and core.jl:271-291 (particle; self included) */
static double sum_at(const orc_system* s, int func, const double* x) {
  double out = 0.0;
  const int64_t key = orc_find_key(s, x);
  for (int c = 0; c < s->n_diff; ++c) {
    const int64_t nk = key + s->key_diff[c];
    if (!(1 <= nk && nk <= s->key_max)) continue;
    for (int64_t e = s->cstart[nk]; e < s->cstart[nk + 1]; ++e) {
      const int64_t q = s->entries[e];
      double d[3];
      const double r = sqrt(dist2(x, s->x[q], d));
      if (r > s->p.h) continue;
      out = out + sum_func(s, func, q, r);
    }
  }
  return out;
}

void orc_sum_point(const orc_system* s, int func, int64_t nq, const double* x, double* out) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < nq; ++i) out[i] = sum_at(s, func, x + 3 * i);
}

void orc_sum_particle(const orc_system* s, int func, int64_t nq, const int64_t* idx,
                      double* out) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < nq; ++i)
    out[i] = sum_at(s, func, s->x[idx[i]]);
}

/* ------------------------------------------------------------- debugging */
int64_t orc_pairs(const orc_system* s, int64_t* pairs, int64_t cap) {
  int64_t cnt = 0;
  for (int64_t p = 0; p < s->n; ++p) {
    const int64_t key = orc_find_key(s, s->x[p]);
    for (int c = 0; c < s->n_diff; ++c) {
      const int64_t nk = key + s->key_diff[c];
      if (!(1 <= nk && nk <= s->key_max)) continue;
      for (int64_t e = s->cstart[nk]; e < s->cstart[nk + 1]; ++e) {
        const int64_t q = s->entries[e];
        double d[3];
        const double r = sqrt(dist2(s->x[p], s->x[q], d));
        if (r > s->p.h || p == q) continue;
        if (cnt < cap) { pairs[2 * cnt] = p; pairs[2 * cnt + 1] = q; }
        ++cnt;
      }
    }
  }
  return cnt;
}

/* ------------------------------------------------- matrix/vector assembly */
/* div_L_lambda! of collapse_dry_implicit.jl:140-145 for particle p (after
 * initialize!: div = L = 0, lambda = 1), neighbours q != p in the
 * reference order; rDkernel is this library's rDW. */
static void div_L_lambda(const orc_system* s, int64_t p, double* div, double* L, double* lam) {
  const double m = s->p.mass, rho = s->p.rho0;
  const double dim = (double)orc_dim(s);
  const int64_t key = orc_find_key(s, s->x[p]);
  double dv = 0.0, l = 0.0, la = 1.0;
  for (int c = 0; c < s->n_diff; ++c) {
    const int64_t nk = key + s->key_diff[c];
    if (!(1 <= nk && nk <= s->key_max)) continue;
    for (int64_t e = s->cstart[nk]; e < s->cstart[nk + 1]; ++e) {
      const int64_t q = s->entries[e];
      double d[3];
      const double r = sqrt(dist2(s->x[p], s->x[q], d));
      if (r > s->p.h || p == q) continue;
      const double rDk = ker_rdw(s, r);
      const double* vp = s->v[p];
      const double* vq = s->v[q];
      /* SmoothedParticles.dot(p.x - q.x, p.v - q.v), algebra.jl:49-51 */
      const double dot = (d[0] * (vp[0] - vq[0]) + d[1] * (vp[1] - vq[1])) + d[2] * (vp[2] - vq[2]);
      dv = dv + ((-dot) * m) * rDk;
      l = l + ((-2.0 * m) / rho) * rDk;
      la = la + (((m / rho) * rDk) * (r * r)) / dim;
    }
  }
  *div = dv;
  *L = l;
  *lam = la;
}

int64_t orc_assemble_matrix(const orc_system* s, int func, double param, int64_t* I, int64_t* J,
                            double* V, int64_t cap) {
  const double H = s->p.h, m = s->p.mass, rho = s->p.rho0;
  const double h2 = H * H;
  int64_t cnt = 0;
  for (int64_t p = 0; p < s->n; ++p) {
    double diag = 0.0;
    if (func == ORC_MAT_PROJECTION) {
      double div, L, lam;
      div_L_lambda(s, p, &div, &L, &lam);
      /* projection_matrix(p, p, 0) */
      diag = s->type[p] == ORC_FLUID ? h2 * L + param * (lam > 0.0 ? lam : 0.0) : h2 * L;
    }
    const int64_t key = orc_find_key(s, s->x[p]);
    for (int c = 0; c < s->n_diff; ++c) {
      const int64_t nk = key + s->key_diff[c];
      if (!(1 <= nk && nk <= s->key_max)) continue;
      for (int64_t e = s->cstart[nk]; e < s->cstart[nk + 1]; ++e) {
        const int64_t q = s->entries[e];
        double d[3];
        const double r = sqrt(dist2(s->x[p], s->x[q], d));
        if (r > H) continue; /* core.jl:210-213: p == q is kept */
        double v;
        if (func == ORC_MAT_KERNEL)
          v = ker_w(s, r);
        else
          v = p == q ? diag : (((2.0 * h2) * m) / rho) * ker_rdw(s, r);
        if (cnt < cap) {
          I[cnt] = p;
          J[cnt] = q;
          V[cnt] = v;
        }
        ++cnt;
      }
    }
  }
  return cnt;
}

void orc_assemble_vector(const orc_system* s, int func, double* out) {
  const double h2 = s->p.h * s->p.h;
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < s->n; ++p) {
    double div, L, lam;
    div_L_lambda(s, p, &div, &L, &lam);
    /* projection_vector: -h^2 p.div / dt */
    out[p] = func == ORC_VEC_PROJECTION ? ((-h2) * div) / s->p.dt : 0.0;
  }
}

/* ------------------------------------------------------ step and initial */
/* collapse_symplectic.jl:186-191 (+ the hydrostatic reference density) */
int64_t orc_init(orc_system* s) {
  int64_t pairs = 0;
  orc_create_cell_list(s);
  orc_apply_unary(s, ORC_OP_RESET_RHO_REF);
  pairs += orc_apply(s, ORC_OP_DENSITY_REF, 1);
  orc_apply_unary(s, ORC_OP_HYDROSTATIC);
  orc_apply_unary(s, ORC_OP_RESET_RHO);
  pairs += orc_apply(s, ORC_OP_DENSITY, 1);
  orc_apply_unary(s, ORC_OP_EOS);
  pairs += orc_apply(s, ORC_OP_WALL_PRESSURE, 0);
  orc_apply_unary(s, ORC_OP_RESET_A);
  pairs += orc_apply(s, ORC_OP_FORCE, 0);
  return pairs;
}

/* collapse_symplectic.jl:170-180 verlet_step! */
int64_t orc_step(orc_system* s, int nsteps) {
  int64_t pairs = 0;
  for (int k = 0; k < nsteps; ++k) {
    orc_apply_unary(s, ORC_OP_KICK);
    orc_apply_unary(s, ORC_OP_DRIFT);
    orc_create_cell_list(s);
    orc_apply_unary(s, ORC_OP_RESET_RHO);
    pairs += orc_apply(s, ORC_OP_DENSITY, 1);
    orc_apply_unary(s, ORC_OP_EOS);
    pairs += orc_apply(s, ORC_OP_WALL_PRESSURE, 0);
    orc_apply_unary(s, ORC_OP_RESET_A);
    pairs += orc_apply(s, ORC_OP_FORCE, 0);
    orc_apply_unary(s, ORC_OP_KICK);
  }
  return pairs;
}

int64_t orc_pair_passes_sample(orc_system* s, int64_t lo, int64_t hi) {
  if (!s->cells_valid) orc_create_cell_list(s);
  if (lo < 0) lo = 0;
  if (hi > s->n) hi = s->n;
  int64_t pairs = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : pairs)
  for (int64_t p = lo; p < hi; ++p) {
    s->rho[p] = 0.0;
    pairs += binary_one(s, ORC_OP_DENSITY, p);
    self_one(s, ORC_OP_DENSITY, p);
  }
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : pairs)
  for (int64_t p = lo; p < hi; ++p) pairs += binary_one(s, ORC_OP_WALL_PRESSURE, p);
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : pairs)
  for (int64_t p = lo; p < hi; ++p) {
    for (int d = 0; d < 3; ++d) { s->a[p][d] = 0.0; s->xs[p][d] = 0.0; }
    pairs += binary_one(s, ORC_OP_FORCE, p);
  }
  return pairs;
}

static void kernel_consts(orc_system* s, int dim, double h) {
  memset(s, 0, sizeof(*s));
  s->kdim = dim;
  s->inv_h = 1.0 / h;
  const double h2 = h * h;
  if (dim == 2) {
    s->cw = 2.228169203286535 / h2;
    s->cr = -44.563384065730695 / (h2 * h2);
  } else {
    s->cw = 3.3422538049298023 / (h2 * h);
    s->cr = -66.84507609859604 / ((h2 * h2) * h);
  }
}

double orc_kernel_w(int dim, double h, double r) {
  orc_system s;
  kernel_consts(&s, dim, h);
  return ker_w(&s, r);
}

double orc_kernel_rdw(int dim, double h, double r) {
  orc_system s;
  kernel_consts(&s, dim, h);
  return ker_rdw(&s, r);
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
