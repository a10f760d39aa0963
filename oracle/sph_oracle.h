/*
 * sph_oracle.h -- CPU oracle for the SmoothedParticles.jl neighbour search and
 * pair loop.  TEST INFRASTRUCTURE ONLY: the GPU library never links, loads or
 * calls this code; only the tests, the smoke check and the CPU-baseline leg of
 * bench.py use it, and only as the checker / the timed CPU arm.
 *
 * What it restates (paths are relative to the SmoothedParticles.jl project):
 *   src/structs.jl:57-92   ParticleSystem constructor: key_phase, key_lim,
 *                          key_max, key_diff (linear neighbour offsets)
 *   src/structs.jl:97-106  find_key (1-based linear cell key, -1 on NaN/Inf)
 *   src/core.jl:8-10       dist = norm(p.x - q.x); src/algebra.jl:49-60 dot/norm
 *   src/core.jl:51-90      create_cell_list!: removal of particles outside the
 *                          domain's bounding box (NaN included), tail-fill
 *                          compaction, cells holding indices in DESCENDING order
 *   src/core.jl:94-161     _apply_binary!/apply_binary!/apply_unary!/apply!:
 *                          traversal in key_diff order, skip r > h or p == q,
 *                          self term appended after all neighbours
 *   src/core.jl:240-291    sum(sys, func, x) and sum(sys, func, p)
 *   src/kernels.jl:108-195 wendland2/rDwendland2/wendland3/rDwendland3
 *   examples/collapse_symplectic.jl:98-143,170-191  operator templates and the
 *                          kick-drift-kick step order
 *   tests/test_collision_2d.jl:63-116  the linear EOS and the P/rho0^2
 *                          pressure force (ORC_EOS_LINEAR), the same step
 *
 * The reference has no Tait EOS, artificial viscosity, XSPH or wall-pressure
 * operator; those are written from the published formulas (Tait/Monaghan
 * 1992 viscosity/Monaghan 1989 XSPH/Adami, Hu & Adams 2012 wall pressure) in
 * the style of the reference's operator templates.
 *
 * Parity status: the reference is Julia and no Julia runtime exists on either
 * machine, and the reference ships no golden outputs for this path.  The oracle
 * is pinned by the reference's own known-answer tests restated in tests/
 * (tests/test_kernels.jl normalisation and derivative checks,
 * tests/test_collision_2d.jl particle-count and energy-drift checks), by the
 * lattice particle counts of src/grids.jl, and by exact hand-derived cases.
 * Bit-level agreement with the Julia runtime is unpinned: kernels.jl is
 * @fastmath, so Julia may legally reassociate it.  The one evaluation order
 * written in sph_oracle.c is the definition both the oracle and the GPU
 * library follow.
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_FLUID = 0, ORC_WALL = 1 };

/* binary (pair) operators */
enum {
  ORC_OP_DENSITY = 1,      /* rho_p     += m W(r)  (fluid p, any q)        */
  ORC_OP_DENSITY_REF = 2,  /* rho_ref_p += m W(r)  (fluid p, any q)        */
  ORC_OP_FORCE = 3,        /* pressure + viscosity + XSPH (fluid p)       */
  ORC_OP_WALL_PRESSURE = 4 /* wall pressure from the fluid (wall p)       */
};
/* unary operators */
enum {
  ORC_OP_RESET_RHO = 10,
  ORC_OP_RESET_RHO_REF = 11,
  ORC_OP_RESET_A = 12,    /* a = 0, xsph = 0                                */
  ORC_OP_EOS = 13,        /* P and the force's P/rho^2 (orc_params.eos)      */
  ORC_OP_KICK = 14,       /* v += dt/2 (a + g)                              */
  ORC_OP_DRIFT = 15,      /* x += dt (v + eps xsph)                         */
  ORC_OP_HYDROSTATIC = 16 /* rho_ref /= (1 + rho0 g (H_col - y)/B)^(1/7)   */
};
/* functions for sum(sys, func, x) */
enum {
  ORC_SUM_DENSITY = 1,  /* m W(r) over all q                        */
  ORC_SUM_KERNEL = 2,   /* W(r) over all q                          */
  ORC_SUM_PRESSURE = 3, /* (m / rho_q) P_q W(r) over fluid q        */
  ORC_SUM_SHEPARD = 4   /* (m / rho_q) W(r) over fluid q            */
};

typedef struct orc_params {
  int32_t dim;           /* 2 or 3 (informational; the geometry decides)    */
  int32_t precision;     /* unused by the oracle (always FP64)              */
  double h;              /* neighbour radius = kernel support H             */
  double domain_min[3];  /* bounding box of the domain                      */
  double domain_max[3];
  double mass;
  double rho0;
  double c0;
  double h_smooth;       /* smoothing length in the viscosity regulariser   */
  double alpha;          /* artificial viscosity coefficient                */
  double eps_xsph;       /* XSPH coefficient                                */
  double gravity[3];
  double dt;
  double col_height;     /* free-surface height for hydrostatic init        */
  int32_t vertical_axis; /* 0-based axis of gravity                         */
  int32_t eos;           /* ORC_EOS_TAIT or ORC_EOS_LINEAR                  */
} orc_params;

/* equation of state (orc_params.eos) and the force's pressure term */
enum {
  ORC_EOS_TAIT = 0,  /* P = B((rho/rho_ref)^7 - 1), B = c0^2 rho0 / 7; P/rho^2 */
  ORC_EOS_LINEAR = 1 /* P = c0^2 (rho - rho_ref); P/rho0^2 -- find_pressure!
                        and internal_force! of tests/test_collision_2d.jl:71-78 */
};

typedef struct orc_system orc_system;

orc_system* orc_create(const orc_params* p);
void orc_destroy(orc_system* s);
int orc_dim(const orc_system* s);
void orc_geometry(const orc_system* s, int64_t key_phase[3], int64_t key_lim[3],
                  int64_t* key_max, int64_t key_diff[27], int32_t* n_diff);
/* Appends n particles (generate_particles! / push!). x, v are n x 3. */
int orc_add_particles(orc_system* s, int64_t n, const double* x, const double* v,
                      const double* rho, const double* rho_ref, const int32_t* type);
int64_t orc_num_particles(const orc_system* s);
/* Copies the state out in the reference's particle order.  Any pointer may be
 * NULL.  oid is the index the particle had when it was added. */
void orc_get_state(const orc_system* s, double* x, double* v, double* a, double* xsph,
                   double* rho, double* rho_ref, double* P, int32_t* type, int64_t* oid);
void orc_set_state(orc_system* s, const double* x, const double* v, const double* a,
                   const double* xsph, const double* rho, const double* rho_ref,
                   const double* P);

int64_t orc_find_key(const orc_system* s, const double x[3]);
void orc_create_cell_list(orc_system* s);
/* apply!(sys, op; self) for built-in operators; returns the number of pair
 * interactions (r <= h, p != q) whose target is a fluid particle. */
int64_t orc_apply(orc_system* s, int op, int self);
void orc_apply_unary(orc_system* s, int op);
/* sum(sys, func, x) at nq points (x is nq x 3) */
void orc_sum_point(const orc_system* s, int func, int64_t nq, const double* x, double* out);
/* sum(sys, func, p) for particles by index (0-based, reference order) */
void orc_sum_particle(const orc_system* s, int func, int64_t nq, const int64_t* idx,
                      double* out);

/* cell keys of all particles in reference order (after create_cell_list) */
void orc_keys(const orc_system* s, int64_t* keys);
/* Every ordered pair (p, q), p != q, r <= h, in the reference's traversal
 * order (p ascending; for each p, key_diff order, descending q).  Writes up to
 * cap pairs and returns the total count. */
int64_t orc_pairs(const orc_system* s, int64_t* pairs, int64_t cap);

/* core.jl:196-225 assemble_matrix / core.jl:175-183 assemble_vector with the
 * built-in functions (the GPU's SPH_MAT_* / SPH_VEC_*).  The matrix entries
 * (I, J, V) are pushed in the reference's loop order: row p, its key_diff
 * cells, each cell's entries, p itself included (r = 0).  Returns the entry
 * count (writes at most cap). */
enum {
  ORC_MAT_KERNEL = 1,     /* W(r)                                              */
  ORC_MAT_PROJECTION = 2  /* collapse_dry_implicit.jl:151-160 (param = C_free) */
};
enum { ORC_VEC_PROJECTION = 1 /* collapse_dry_implicit.jl:162-164, div by div_L_lambda! */ };
int64_t orc_assemble_matrix(const orc_system* s, int func, double param, int64_t* I, int64_t* J,
                            double* V, int64_t cap);
void orc_assemble_vector(const orc_system* s, int func, double* out);

/* Initialisation of the dam-break state (collapse_symplectic.jl:186-191 plus
 * the hydrostatic reference density) and the kick-drift-kick step
 * (collapse_symplectic.jl:170-180).  Both return fluid-target pair counts. */
int64_t orc_init(orc_system* s);
int64_t orc_step(orc_system* s, int nsteps);
/* Same as one step but only the pair passes over targets in [lo, hi) are
 * evaluated (a bounded sample used by the CPU baseline).  Returns pairs. */
int64_t orc_pair_passes_sample(orc_system* s, int64_t lo, int64_t hi);

int orc_num_threads(void);

/* The kernel functions themselves (kernels.jl:108-195) for a given dimension
 * and support radius, in the oracle's evaluation order. */
double orc_kernel_w(int dim, double h, double r);
double orc_kernel_rdw(int dim, double h, double r);

#ifdef __cplusplus
}
#endif
#endif
