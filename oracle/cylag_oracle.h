/*
 * cylag_oracle.h -- CPU restatement of CyLag's per-particle time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU step is checked
 * against; the product never links it.  Every function follows the
 * reference Cython source, cited as file:line relative to the CyLag tree.
 * It is itself pinned against the compiled reference through the golden
 * fixtures in tests/golden/.
 *
 * Semantics that differ from the unmodified reference, by design:
 *  - per-particle PCG32 streams: particle i draws from its own (state, inc)
 *    pair, seeded pcg32_seed(seed, tag).  The reference draws from one global
 *    generator in particle order (cylag/lsm/random_utils.pyx:16-20); running
 *    the reference one particle at a time with pcg32_seed(seed, tag) before
 *    each particle reproduces this convention exactly.
 *  - the localization fallback (reference: scipy cKDTree candidates,
 *    cylag/geom/xylocalizer.pyx:200-286) returns the lowest-index triangle
 *    containing the point; both agree unless the point lies exactly on an
 *    edge shared by two triangles.
 *  - deleted particles are retagged maxtag+1, maxtag+2, ... in particle-index
 *    order by a serial pass after the step (the reference retags inside the
 *    loop, cylag/core/lagrangian_particle_set.pyx:786-788 -- same order).
 */
#ifndef CYLAG_ORACLE_H
#define CYLAG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nv, nt, ne;
    const double *x, *y;          /* [nv] */
    const int32_t *tri;           /* [nt][3] */
    const double *gradx, *grady, *det; /* [nt][3] */
    const int32_t *edges;         /* [ne][2] */
    const int32_t *triedge;       /* [nt][3] */
    const int32_t *edgetri;       /* [ne][2] */
    const int32_t *edge_labels;   /* [ne] */
    /* optional bucket grid (NULL gstart: exhaustive search) */
    double gx0, gy0, ginv;
    int gnx, gny;
    const int32_t *gstart, *gtris;
} cgo_mesh;

typedef struct {
    int dim;          /* field-set dimension (2 or 3) */
    int nlayers;
    int npoints;
    int frozen;       /* frozen_hydro */
    int prev_valid;   /* previous-step temps meaningful (acceleration) */
    /* time-interpolated node fields, each [npoints*nlayers]; NULL if absent */
    const double *zs, *ux, *uy, *uz, *kt, *ep, *zb;
    /* previous-step temps (acceleration, LSM3) */
    const double *z0, *u0, *v0, *w0;
} cgo_fields;

typedef struct {
    /* Parameters (cylag/cylag_dico.py:9-51) */
    int model, time_scheme, rng_method, diffusion_model;
    int diffusion_lsm2_option, lsm3_edge_opt;
    int boundary_conditions, bc_type, max_wall_rebounds, bnd_statistics;
    int particle_velocity_init;
    double dt, time;
    double nux, nuz, sigc;
    double tl_h, tl_v;                  /* diffusion_lsm3_tl_horizontal/vertical */
    double damp_coef, roughness_deg, strand_prob;
    /* particle-set properties (cylag/core/lagrangian_particle_set.pyx:158-261) */
    int pdim;
    double rho0, density;
    int drag_model; double drag_coef;
    int added_mass; double added_mass_coef;
    int buoy_model; double buoy_value;
    double a0c, a1c, a2c, a3c;
    /* field-set friction law of the pseudo-3D log-law correction
     * (eulerian_field_set.pyx:125-138, 1957-1993) */
    int friction_model; double friction_coef;
    /* LagrangianParticleSet.compute_depth (solver.pyx:526-538) */
    int compute_depth;
} cgo_params;

typedef struct {
    int n;
    double *pos, *vel, *fvs;            /* [n][pdim] */
    double *last_pos, *last_vel;        /* [n][pdim] */
    int32_t *tri, *last_tri, *lowerlayer, *inactive, *tag;
    double *diameter, *volume;
    uint64_t *rng_state, *rng_inc;      /* per-particle PCG32 */
    double *depth;                      /* [n] or NULL (compute_depth) */
} cgo_particles;

/* ---- RNG (cylag/lsm/random_utils.pyx) ---- */
void cgo_pcg32_seed(uint64_t *state, uint64_t *inc, uint64_t seed, uint64_t stream);
void cgo_pcg32_advance(uint64_t *state, uint64_t inc, uint64_t delta);
/* fill out[0..n) with draws of kind: 0 uniform, 1 ziggurat, 2 polar single,
 * 3 pair(method) flattened (2n values), 4 single(method) */
void cgo_rng_draws(uint64_t seed, uint64_t stream, int kind, int method,
                   int64_t n, double *out);
void cgo_ziggurat_tables(uint32_t *kn, double *wn, double *fn);

/* ---- geometry (cylag/geom) ---- */
int cgo_point_in_tri(const cgo_mesh *m, int k, double x, double y);
int cgo_locate_exhaustive(const cgo_mesh *m, double x, double y);
int cgo_locate(const cgo_mesh *m, double x, double y);
void cgo_xy_localize(const cgo_mesh *m, int k, double p0x, double p0y,
                     double x, double y, int *new_k, int *bnd_j);
int cgo_lower_layer_index(int nlayers, double zs, double zb, double z);

/* ---- fields (cylag/core/eulerian_field_set.pyx) ---- */
void cgo_time_interp(int64_t size, double tf, const double *f0,
                     const double *f1, double *out);

/* ---- step (cylag/core/solver.pyx:459-549) ----
 * Advances particles [i0, i1) by one step.  bnd_stats may be NULL.
 * Returns the number of particles deleted (tags set to -1; call
 * cgo_retag afterwards).  Particles with tri == -2 are initialized first. */
int cgo_step_range(const cgo_mesh *m, const cgo_fields *f, const cgo_params *p,
                   cgo_particles *s, int i0, int i1, int32_t *bnd_stats);
/* Same over all particles with nthreads OpenMP threads. */
int cgo_step(const cgo_mesh *m, const cgo_fields *f, const cgo_params *p,
             cgo_particles *s, int32_t *bnd_stats, int nthreads);
/* Serial retag pass: tag == -1 on an inactive particle -> ++maxtag. */
int cgo_retag(cgo_particles *s, int maxtag);
/* Solver.initialize_particle_state (cylag/core/solver.pyx:238-379) for
 * particles [i0, i1) that are active. Returns number deleted. */
int cgo_init_range(const cgo_mesh *m, const cgo_fields *f, const cgo_params *p,
                   cgo_particles *s, int i0, int i1);

/* Number of particles, since the previous call, whose step or
 * initialization met a condition on which the reference raises ValueError
 * (interpolation outside the mesh or the column, non-finite LSM2/LSM3
 * coefficients, ...); their state is then unspecified.  Resets the count. */
int cgo_take_errors(void);
void cgo_set_stranding(int on);
int cgo_set_sections(int n, const double *seg);
void cgo_take_section_counts(int32_t *out);
int cgo_take_stranded(double *out, int cap);

#ifdef __cplusplus
}
#endif
#endif
