/*
 * cylag_oracle.c -- CPU restatement of CyLag's per-particle time step.
 *
 * TEST INFRASTRUCTURE ONLY (see cylag_oracle.h).  Plain C, scalar, FP64,
 * compiled with -ffp-contract=off so that every multiply and add rounds
 * separately, exactly as the reference's Cython-generated C does under gcc
 * -O2 on x86-64.  Expressions keep the reference's evaluation order.
 */
#include "cylag_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* cylag/core/constants.pyx:1-75 */
#define EPSILON 1.e-16
#define EPSILON_LSM2 1.e-8
#define EPSILON_LSM3 1.e-8
#define EPSILON_REBOUND 1.e-8
#define LSM3_CLIP_STEP 1.e-4
#define DEG_TO_RAD 0.017453292519943295
#define TWO_SQRT3 3.4641016151377544
#define BND_WALL_REF 0
#define BND_OPEN_REF 1
#define PART_LOC_O (-1)
#define PART_LOC_B (-2)
#define PART_LOC_A (-3)
#define GRAV 9.80665
#define NU0 1.3e-6
#define C0KOLM 1.2
#define CMU 0.09
#define KAPPA 0.41
#define DBL_EPS 2.220446049250313e-16

/* ======================================================================
 * PCG32 + normal variates (cylag/lsm/random_utils.pyx)
 * ====================================================================== */
typedef struct { uint64_t state, inc; } rng_t;

/* random_utils.pyx:22-28 */
static inline uint32_t pcg_next(rng_t *r) {
    uint64_t old = r->state;
    r->state = old * 6364136223846793005ULL + r->inc;
    uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((32 - rot) & 31));
}

/* random_utils.pyx:30-37 */
void cgo_pcg32_seed(uint64_t *state, uint64_t *inc, uint64_t seed, uint64_t stream) {
    rng_t r;
    r.state = 0;
    r.inc = (stream << 1) | 1;
    pcg_next(&r);
    r.state += seed;
    pcg_next(&r);
    *state = r.state;
    *inc = r.inc;
}

/* random_utils.pyx:39-53 */
void cgo_pcg32_advance(uint64_t *state, uint64_t inc, uint64_t delta) {
    uint64_t acc_mult = 1, acc_plus = 0;
    uint64_t cur_mult = 6364136223846793005ULL, cur_plus = inc;
    while (delta > 0) {
        if (delta & 1) {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1;
    }
    *state = acc_mult * (*state) + acc_plus;
}

/* random_utils.pyx:55-67 */
static inline double rng_uniform(rng_t *r) {
    uint32_t u = pcg_next(r);
    return u * (1.0 / 4294967296.0);
}

/* random_utils.pyx:72-88 */
static double rng_polar_single(rng_t *r) {
    double x1 = 0., x2, w = 2.0;
    while (w >= 1.0 || w == 0.0) {
        x1 = 2.0 * rng_uniform(r) - 1.0;
        x2 = 2.0 * rng_uniform(r) - 1.0;
        w = x1 * x1 + x2 * x2;
    }
    w = sqrt((-2.0 * log(w)) / w);
    return x1 * w;
}

/* random_utils.pyx:90-108 */
static void rng_polar_pair(rng_t *r, double *a, double *b) {
    double x1 = 0., x2 = 0., w = 2.0;
    while (w >= 1.0 || w == 0.0) {
        x1 = 2.0 * rng_uniform(r) - 1.0;
        x2 = 2.0 * rng_uniform(r) - 1.0;
        w = x1 * x1 + x2 * x2;
    }
    w = sqrt((-2.0 * log(w)) / w);
    *a = x1 * w;
    *b = x2 * w;
}

/* Ziggurat tables, random_utils.pyx:113-149 (Marsaglia & Tsang 2000, 128
 * layers).  Built once with the host libm, as the reference does at import. */
static uint32_t zkn[128];
static double zwn[128], zfn[128];
static int ztables_ready = 0;
static const double ZIG_R = 3.442619855899;

static void zig_init(void) {
    if (ztables_ready) return;
    double m1 = 2147483648.0, dn = 3.442619855899, tn = dn;
    double vn = 9.91256303526217e-3;
    double q = vn / exp(-0.5 * dn * dn);
    zkn[0] = (uint32_t)((dn / q) * m1);
    zkn[1] = 0;
    zwn[0] = q / m1;
    zwn[127] = dn / m1;
    zfn[0] = 1.0;
    zfn[127] = exp(-0.5 * dn * dn);
    for (int i = 126; i >= 1; i--) {
        dn = sqrt(-2.0 * log(vn / dn + exp(-0.5 * dn * dn)));
        zkn[i + 1] = (uint32_t)((dn / tn) * m1);
        tn = dn;
        zfn[i] = exp(-0.5 * dn * dn);
        zwn[i] = dn / m1;
    }
    ztables_ready = 1;
}

void cgo_ziggurat_tables(uint32_t *kn, double *wn, double *fn) {
    zig_init();
    memcpy(kn, zkn, sizeof zkn);
    memcpy(wn, zwn, sizeof zwn);
    memcpy(fn, zfn, sizeof zfn);
}

/* random_utils.pyx:154-194 */
static double rng_ziggurat(rng_t *r) {
    for (;;) {
        int32_t hz = (int32_t)pcg_next(r);
        uint32_t iz = (uint32_t)hz & 127;
        /* c_abs(INT_MIN) stays INT_MIN, i.e. 2^31 once cast (line 173) */
        uint32_t ahz = hz < 0 ? (uint32_t)0 - (uint32_t)hz : (uint32_t)hz;
        if (ahz < zkn[iz]) return hz * zwn[iz];
        if (iz == 0) {
            for (;;) {
                double x = -log(rng_uniform(r)) * 0.2904764;
                double y = -log(rng_uniform(r));
                if (y + y >= x * x) return hz > 0 ? ZIG_R + x : -ZIG_R - x;
            }
        }
        double x = hz * zwn[iz];
        if (zfn[iz] + rng_uniform(r) * (zfn[iz - 1] - zfn[iz]) < exp(-0.5 * x * x))
            return x;
    }
}

/* random_utils.pyx:202-233 */
static void rng_pair(rng_t *r, int method, double *a, double *b) {
    if (method == 1) {
        *a = (rng_uniform(r) - 0.5) * TWO_SQRT3;
        *b = (rng_uniform(r) - 0.5) * TWO_SQRT3;
    } else if (method == 2) {
        *a = rng_ziggurat(r);
        *b = rng_ziggurat(r);
    } else {
        rng_polar_pair(r, a, b);
    }
}

/* random_utils.pyx:235-263 */
static double rng_single(rng_t *r, int method) {
    if (method == 1) return (rng_uniform(r) - 0.5) * TWO_SQRT3;
    if (method == 2) return rng_ziggurat(r);
    return rng_polar_single(r);
}

void cgo_rng_draws(uint64_t seed, uint64_t stream, int kind, int method,
                   int64_t n, double *out) {
    rng_t r;
    zig_init();
    cgo_pcg32_seed(&r.state, &r.inc, seed, stream);
    for (int64_t i = 0; i < n; i++) {
        switch (kind) {
        case 0: out[i] = rng_uniform(&r); break;
        case 1: out[i] = rng_ziggurat(&r); break;
        case 2: out[i] = rng_polar_single(&r); break;
        case 3: rng_pair(&r, method, &out[2 * i], &out[2 * i + 1]); break;
        default: out[i] = rng_single(&r, method); break;
        }
    }
}

/* ======================================================================
 * Geometry (cylag/geom/utils.pyx, intersections.pyx, xylocalizer.pyx)
 * ====================================================================== */

/* utils.pyx:332-361 */
static inline double pintri(double x, double y, double xa, double ya,
                            double xb, double yb, double xc, double yc) {
    return ((xb - xa) * (y - ya) - (x - xa) * (yb - ya))
         * ((x - xa) * (yc - ya) - (xc - xa) * (y - ya));
}

/* utils.pyx:363-385 */
static inline int point_in_triangle_dotp(double x, double y, double x0, double y0,
                                         double x1, double y1, double x2, double y2) {
    return pintri(x, y, x0, y0, x1, y1, x2, y2) >= 0
        && pintri(x, y, x1, y1, x2, y2, x0, y0) >= 0
        && pintri(x, y, x2, y2, x0, y0, x1, y1) >= 0;
}

/* xylocalizer.pyx:126-167 (k == -1 reads the last triangle: wraparound) */
int cgo_point_in_tri(const cgo_mesh *m, int k, double x, double y) {
    int kk = k < 0 ? k + m->nt : k;
    int v0 = m->tri[3 * kk], v1 = m->tri[3 * kk + 1], v2 = m->tri[3 * kk + 2];
    if (point_in_triangle_dotp(x, y, m->x[v0], m->y[v0], m->x[v1], m->y[v1],
                               m->x[v2], m->y[v2]))
        return k;
    return -1;
}

/* utils.pyx:228-252 */
static inline int orientation(double v0x, double v0y, double v1x, double v1y,
                              double v2x, double v2y) {
    double delta = (v0y - v1y) * (v2x - v0x) - (v0x - v1x) * (v2y - v0y);
    if (delta == 0.) return 0;
    else if (delta > 0.) return 1;
    return 2;
}

/* utils.pyx:282-303 */
static inline int on_segment(double v0x, double v0y, double v1x, double v1y,
                             double v2x, double v2y) {
    return v2x <= fmax(v1x, v0x) && v2x >= fmin(v1x, v0x)
        && v2y <= fmax(v1y, v0y) && v2y >= fmin(v1y, v0y);
}

/* intersections.pyx:106-148 */
static int intersec2d(double p0x, double p0y, double p1x, double p1y,
                      double s0x, double s0y, double s1x, double s1y) {
    int o1 = orientation(p0x, p0y, p1x, p1y, s0x, s0y);
    int o2 = orientation(p0x, p0y, p1x, p1y, s1x, s1y);
    int o3 = orientation(s0x, s0y, s1x, s1y, p0x, p0y);
    int o4 = orientation(s0x, s0y, s1x, s1y, p1x, p1y);
    if (o1 != o2 && o3 != o4) return 1;
    if (o1 == 0 && on_segment(p0x, p0y, p1x, p1y, s0x, s0y)) return 1;
    if (o2 == 0 && on_segment(p0x, p0y, p1x, p1y, s1x, s1y)) return 1;
    if (o3 == 0 && on_segment(s0x, s0y, s1x, s1y, p0x, p0y)) return 1;
    if (o4 == 0 && on_segment(s0x, s0y, s1x, s1y, p1x, p1y)) return 1;
    return 0;
}

/* Exhaustive search, lowest index first (stands in for the cKDTree
 * candidate search of xylocalizer.pyx:200-286, same result off edges). */
int cgo_locate_exhaustive(const cgo_mesh *m, double x, double y) {
    for (int k = 0; k < m->nt; k++)
        if (cgo_point_in_tri(m, k, x, y) != -1) return k;
    return -1;
}

/* Lowest-index triangle containing the point, found through the bucket
 * grid when one is given (each bucket lists, in increasing id, every triangle
 * whose padded bounding box touches it), else by exhaustive search. */
int cgo_locate(const cgo_mesh *m, double x, double y) {
    if (!m->gstart) return cgo_locate_exhaustive(m, x, y);
    double fx = floor((x - m->gx0) * m->ginv), fy = floor((y - m->gy0) * m->ginv);
    if (!(fx >= 0.)) fx = 0.;
    if (!(fy >= 0.)) fy = 0.;
    int cx = fx > (double)(m->gnx - 1) ? m->gnx - 1 : (int)fx;
    int cy = fy > (double)(m->gny - 1) ? m->gny - 1 : (int)fy;
    int c = cy * m->gnx + cx;
    for (int j = m->gstart[c]; j < m->gstart[c + 1]; j++)
        if (cgo_point_in_tri(m, m->gtris[j], x, y) != -1) return m->gtris[j];
    return -1;
}

/* xylocalizer.pyx:338-435.  k == -1 (a particle whose element was set to
 * "outside" by an aborted Runge-Kutta stage) reads the last triangle's row
 * (numpy wraparound) but compares as -1, as the reference does. */
static void path_walk(const cgo_mesh *m, int k, double p0x, double p0y,
                      double x, double y, int *new_k_out, int *bnd_out) {
    int new_k = -1, niter = 0, niter_max = 50, intersected_edge = -1;
    while (new_k == -1 && niter <= niter_max) {
        int intersects = 0;
        int row = k < 0 ? k + m->nt : k;
        for (int i = 0; i < 3; i++) {
            int j = m->triedge[3 * row + i];
            if (j == intersected_edge) continue;
            int i0 = m->edges[2 * j], i1 = m->edges[2 * j + 1];
            if (intersec2d(p0x, p0y, x, y, m->x[i0], m->y[i0], m->x[i1], m->y[i1])) {
                intersects = 1;
                int k0 = m->edgetri[2 * j], k1 = m->edgetri[2 * j + 1];
                int kn = (k0 == k) ? k1 : k0;
                if (kn == -1) { *new_k_out = -1; *bnd_out = j; return; }
                new_k = cgo_point_in_tri(m, kn, x, y);
                if (new_k != -1) { *new_k_out = new_k; *bnd_out = -1; return; }
                k = kn;
                intersected_edge = j;
                break;
            }
        }
        if (intersects == 0) {
            new_k = cgo_point_in_tri(m, k, x, y);
            *new_k_out = (new_k == -1) ? -1 : k;
            *bnd_out = -1;
            return;
        }
        niter += 1;
    }
    *new_k_out = new_k;
    *bnd_out = -1;
}

/* xylocalizer.pyx:27-124, method 3 (path search, then global fallback) */
void cgo_xy_localize(const cgo_mesh *m, int k, double p0x, double p0y,
                     double x, double y, int *new_k, int *bnd_j) {
    int nk = cgo_point_in_tri(m, k, x, y);
    *bnd_j = -1;
    if (nk != -1) { *new_k = nk; return; }
    path_walk(m, k, p0x, p0y, x, y, &nk, bnd_j);
    if (nk == -1 && *bnd_j == -1) nk = cgo_locate(m, x, y);
    *new_k = nk;
}

/* zlocalizer.pyx:51-71 */
int cgo_lower_layer_index(int nlayers, double zs, double zb, double z) {
    if (nlayers == 1) return 0;
    double hl = (zs - zb) / (nlayers - 1);
    if (!(hl > 0.)) return 0;
    double findex = floor((z - zb) / hl);
    if (!(findex >= 0.)) return 0;
    if (!(findex <= (double)(nlayers - 2))) return nlayers - 2;
    return (int)findex;
}

/* ======================================================================
 * Field interpolation (cylag/core/eulerian_field_set.pyx)
 * ====================================================================== */

/* eulerian_field_set.pyx:930-938 */
void cgo_time_interp(int64_t size, double tf, const double *f0,
                     const double *f1, double *out) {
    for (int64_t i = 0; i < size; i++)
        out[i] = tf * f0[i] + (1. - tf) * f1[i];
}

typedef struct { int i0, i1, i2; double f0, f1, f2; } p1_t;

/* eulerian_field_set.pyx:1043-1052 (P1 factors) */
static inline p1_t p1_factors(const cgo_mesh *m, int k, double x, double y) {
    p1_t p;
    const double *d = m->det + 3 * k, *gx = m->gradx + 3 * k, *gy = m->grady + 3 * k;
    p.f0 = d[0] + x * gx[0] + y * gy[0];
    p.f1 = d[1] + x * gx[1] + y * gy[1];
    p.f2 = d[2] + x * gx[2] + y * gy[2];
    p.i0 = m->tri[3 * k]; p.i1 = m->tri[3 * k + 1]; p.i2 = m->tri[3 * k + 2];
    return p;
}

static inline double p1_eval(const double *fld, int off, const p1_t *p) {
    return fld[off + p->i0] * p->f0 + fld[off + p->i1] * p->f1 + fld[off + p->i2] * p->f2;
}

/* eulerian_field_set.pyx:994-1055: field at layer l (3D) or the 2D field */
static double interp_field_2d(const cgo_mesh *m, const cgo_fields *f,
                              const double *fld, int k, int l, double x, double y) {
    p1_t p = p1_factors(m, k, x, y);
    int off = (f->dim == 2) ? 0 : l * f->npoints;
    return p1_eval(fld, off, &p);
}

/* eulerian_field_set.pyx:1057-1115 */
static void interp_velocity_2d(const cgo_mesh *m, const cgo_fields *f, int k,
                               double x, double y, double *u, double *v) {
    p1_t p = p1_factors(m, k, x, y);
    *u = p1_eval(f->ux, 0, &p);
    *v = p1_eval(f->uy, 0, &p);
}

/* eulerian_field_set.pyx:1289-1394 (zlocalize == 0: lowerlayer given) */
static int interp_velocity_3d(const cgo_mesh *m, const cgo_fields *f, int k, int ll,
                              double x, double y, double z,
                              double *u, double *v, double *w) {
    p1_t p = p1_factors(m, k, x, y);
    if (ll == PART_LOC_B || ll == PART_LOC_A) return -1;
    int jl = ll * f->npoints, ju = (ll + 1) * f->npoints;
    double zlp = p1_eval(f->zs, jl, &p);
    double zup = p1_eval(f->zs, ju, &p);
    double dz = zlp - zup;
    if (fabs(dz) < EPSILON) return -2;
    double zf0 = (z - zup) / dz;
    double zf1 = (zlp - z) / dz;
    *u = zf0 * p1_eval(f->ux, jl, &p) + zf1 * p1_eval(f->ux, ju, &p);
    *v = zf0 * p1_eval(f->uy, jl, &p) + zf1 * p1_eval(f->uy, ju, &p);
    *w = zf0 * p1_eval(f->uz, jl, &p) + zf1 * p1_eval(f->uz, ju, &p);
    return 0;
}

/* eulerian_field_set.pyx:1117-1182 */
static int z_localize(const cgo_mesh *m, const cgo_fields *f, int k,
                      double x, double y, double z) {
    if (k == -1) return PART_LOC_O;
    p1_t p = p1_factors(m, k, x, y);
    double zbp, zsp;
    int nl = f->nlayers, ll;
    if (f->dim == 2) {
        zbp = p1_eval(f->zb, 0, &p);
        zsp = p1_eval(f->zs, 0, &p);
        ll = 0;
    } else {
        zbp = p1_eval(f->zs, 0, &p);
        zsp = p1_eval(f->zs, (nl - 1) * f->npoints, &p);
        ll = cgo_lower_layer_index(nl, zsp, zbp, z);
    }
    if (z < zbp) ll = PART_LOC_B;
    else if (z > zsp) ll = PART_LOC_A;
    return ll;
}

/* eulerian_field_set.pyx:1995-1997 */
static inline double keps_K(double k, double eps, double fac) {
    return fac * k * k / fmax(eps, EPSILON);
}

/* eulerian_field_set.pyx:1644-1763 */
static int interp_diffusivity_gradient(const cgo_mesh *m, const cgo_fields *f,
                                       int k, int ll, double x, double y, double z,
                                       double sigc, double *K, double *dKdx,
                                       double *dKdy, double *dKdz) {
    double fac = CMU / sigc;
    p1_t p = p1_factors(m, k, x, y);
    const double *gx = m->gradx + 3 * k, *gy = m->grady + 3 * k;
    const double *kt = f->kt, *ep = f->ep;
    if (f->dim == 2) {
        double kn0 = keps_K(kt[p.i0], ep[p.i0], fac);
        double kn1 = keps_K(kt[p.i1], ep[p.i1], fac);
        double kn2 = keps_K(kt[p.i2], ep[p.i2], fac);
        double Kp = kn0 * p.f0 + kn1 * p.f1 + kn2 * p.f2;
        *dKdx = kn0 * gx[0] + kn1 * gx[1] + kn2 * gx[2];
        *dKdy = kn0 * gy[0] + kn1 * gy[1] + kn2 * gy[2];
        *dKdz = 0.;
        *K = fmax(0., Kp);
        return 0;
    }
    if (ll == PART_LOC_B || ll == PART_LOC_A) return -1;
    int jl = ll * f->npoints, ju = (ll + 1) * f->npoints;
    const double *el = f->zs;
    double kn0 = keps_K(kt[jl + p.i0], ep[jl + p.i0], fac);
    double kn1 = keps_K(kt[jl + p.i1], ep[jl + p.i1], fac);
    double kn2 = keps_K(kt[jl + p.i2], ep[jl + p.i2], fac);
    double Kl = kn0 * p.f0 + kn1 * p.f1 + kn2 * p.f2;
    double gxl = kn0 * gx[0] + kn1 * gx[1] + kn2 * gx[2];
    double gyl = kn0 * gy[0] + kn1 * gy[1] + kn2 * gy[2];
    double zlp = p1_eval(el, jl, &p);
    double zlx = el[jl + p.i0] * gx[0] + el[jl + p.i1] * gx[1] + el[jl + p.i2] * gx[2];
    double zly = el[jl + p.i0] * gy[0] + el[jl + p.i1] * gy[1] + el[jl + p.i2] * gy[2];
    kn0 = keps_K(kt[ju + p.i0], ep[ju + p.i0], fac);
    kn1 = keps_K(kt[ju + p.i1], ep[ju + p.i1], fac);
    kn2 = keps_K(kt[ju + p.i2], ep[ju + p.i2], fac);
    double Ku = kn0 * p.f0 + kn1 * p.f1 + kn2 * p.f2;
    double gxu = kn0 * gx[0] + kn1 * gx[1] + kn2 * gx[2];
    double gyu = kn0 * gy[0] + kn1 * gy[1] + kn2 * gy[2];
    double zup = p1_eval(el, ju, &p);
    double zux = el[ju + p.i0] * gx[0] + el[ju + p.i1] * gx[1] + el[ju + p.i2] * gx[2];
    double zuy = el[ju + p.i0] * gy[0] + el[ju + p.i1] * gy[1] + el[ju + p.i2] * gy[2];
    double dz = zup - zlp;
    if (fabs(dz) < EPSILON) return -2;
    double s = (z - zlp) / dz;
    double Kp = (1. - s) * Kl + s * Ku;
    *dKdz = (Ku - Kl) / dz;
    *dKdx = (1. - s) * gxl + s * gxu - *dKdz * ((1. - s) * zlx + s * zux);
    *dKdy = (1. - s) * gyl + s * gyu - *dKdz * ((1. - s) * zly + s * zuy);
    *K = fmax(0., Kp);
    return 0;
}

/* ======================================================================
 * Particle-set helpers (cylag/core/lagrangian_particle_set.pyx)
 * ====================================================================== */

/* lagrangian_particle_set.pyx:834-890 (model_hr = 0 from update_state_lsm1) */
static double buoyancy_velocity(const cgo_params *p, double dp, int model_hr, double rho0) {
    double rhop = p->density, Cd = p->drag_coef, s = rhop / rho0, wb;
    if (p->buoy_model == 0) return p->buoy_value;
    if (dp < 1.e-4) {
        wb = fabs(s - 1.) * (GRAV * (dp * dp)) / (18. * NU0);
    } else if (dp > 1.e-3) {
        if (model_hr == 0) wb = sqrt(fabs(s - 1.) * (4. * dp * GRAV) / (3. * Cd));
        else wb = 1.1 * sqrt((s - 1.) * GRAV * dp);
    } else {
        wb = (10. * NU0 / dp) * (sqrt(1. + fabs(s - 1.) * GRAV * pow(dp, 3.0) / (100. * (NU0 * NU0))) - 1.);
    }
    if (s > 1.) wb *= -1.;
    return wb;
}

/* lagrangian_particle_set.pyx:766-788 (tag reassigned by cgo_retag) */
static void delete_single(cgo_particles *s, int pdim, int i) {
    if (s->inactive[i] != 0) return;
    s->inactive[i] = 1;
    s->diameter[i] = 0.;
    s->volume[i] = 0.;
    for (int d = 0; d < pdim; d++) {
        s->pos[i * pdim + d] = 0.;
        s->vel[i * pdim + d] = 0.;
        s->fvs[i * pdim + d] = 0.;
        s->last_pos[i * pdim + d] = 0.;
        s->last_vel[i * pdim + d] = 0.;
    }
    if (s->depth) s->depth[i] = 0.;
    s->tri[i] = -1;
    s->lowerlayer[i] = 0;
    s->last_tri[i] = -1;
    s->tag[i] = -1;
}

int cgo_retag(cgo_particles *s, int maxtag) {
    for (int i = 0; i < s->n; i++)
        if (s->inactive[i] && s->tag[i] == -1) s->tag[i] = ++maxtag;
    return maxtag;
}

/* ======================================================================
 * LSM1 (cylag/lsm/update_state_lsm1.pyx)
 * ====================================================================== */

typedef struct {
    const cgo_mesh *m;
    const cgo_fields *f;
    const cgo_params *p;
    cgo_particles *s;
    int i, pd;
    rng_t rng;
    int err;
} ctx_t;

#define POS(c, d) ((c)->s->pos[(c)->i * (c)->pd + (d)])
#define VEL(c, d) ((c)->s->vel[(c)->i * (c)->pd + (d)])
#define FVS(c, d) ((c)->s->fvs[(c)->i * (c)->pd + (d)])
#define LPOS(c, d) ((c)->s->last_pos[(c)->i * (c)->pd + (d)])
#define LVEL(c, d) ((c)->s->last_vel[(c)->i * (c)->pd + (d)])

static double cpow_re(double x, double y);

/* eulerian_field_set.pyx:1957-1993: friction coefficient of the depth h */
static double friction_calc(const cgo_params *p, double h) {
    double fc = p->friction_coef;
    switch (p->friction_model) {
    case 0: return 2. * GRAV / (fc * fc);                                     /* Chezy */
    case 1: return 2. * GRAV / (fc * fc) / cpow_re(fmax(EPSILON, h), 1. / 3.);  /* Strickler */
    case 2: return 2. * GRAV * (fc * fc) / cpow_re(fmax(EPSILON, h), 1. / 3.);  /* Manning */
    default: {                                                                /* Nikuradse */
        double aux = h * 11.036 / fc;
        if (!(aux > 1.001)) aux = 1.001;
        double q = log(aux) / KAPPA;
        return 2. / (q * q);
    }
    }
}

/* eulerian_field_set.pyx:1887-1955: vertical velocity w and horizontal
 * log-law factor of a 3D particle on 2D fields (pseudo-3D) */
static void pseudo_3d_corrections(ctx_t *c, int k, double x, double y, double z, double dt,
                                  double ux, double uy, double *w, double *hor) {
    const cgo_mesh *m = c->m;
    const cgo_fields *f = c->f;
    p1_t p = p1_factors(m, k, x, y);
    const double *gx = m->gradx + 3 * k, *gy = m->grady + 3 * k;
    double zs = p1_eval(f->zs, 0, &p);
    double zb = p1_eval(f->zb, 0, &p);
    double h = fmax(EPSILON, zs - zb);
    double sigma = fmin(1., fmax(0., (z - zb) / h));
    double Cf = friction_calc(c->p, h);
    double z0 = fmax(EPSILON, h * exp(-(1. + KAPPA / sqrt(Cf / 2.))));
    double hh = (z - zb <= z0) ? 0.0 : log((z - zb) / z0) / (log(h / z0) - 1.);
    double uc = ux * hh, vc = uy * hh;
    double dzsdx = f->zs[p.i0] * gx[0] + f->zs[p.i1] * gx[1] + f->zs[p.i2] * gx[2];
    double dzsdy = f->zs[p.i0] * gy[0] + f->zs[p.i1] * gy[1] + f->zs[p.i2] * gy[2];
    double dzbdx = f->zb[p.i0] * gx[0] + f->zb[p.i1] * gx[1] + f->zb[p.i2] * gx[2];
    double dzbdy = f->zb[p.i0] * gy[0] + f->zb[p.i1] * gy[1] + f->zb[p.i2] * gy[2];
    /* eulerian_field_set.pyx:1581-1642 */
    double dzsdt = 0.;
    if (!(f->frozen == 1 || !f->prev_valid)) {
        double z0p = p1_eval(f->z0, 0, &p);
        dzsdt = (zs - z0p) / dt;
    }
    *w = (1. - sigma) * (uc * dzbdx + vc * dzbdy) + sigma * (dzsdt + uc * dzsdx + vc * dzsdy);
    *hor = hh;
}

/* mean velocity at (k, ll, x, y, z), update_state_lsm1.pyx:144-163 */
static void lsm1_velocity(ctx_t *c, int k, int ll, double x, double y, double z,
                          double *ux, double *uy, double *uz) {
    if (c->f->dim == 2) {
        interp_velocity_2d(c->m, c->f, k, x, y, ux, uy);
        *uz = 0.;
        if (c->pd == 3) {
            /* pseudo-3D corrections (update_state_lsm1.pyx:156-162) */
            double w, hor;
            pseudo_3d_corrections(c, k, x, y, z, c->p->dt, *ux, *uy, &w, &hor);
            *uz += w;
            *ux *= hor;
            *uy *= hor;
        }
    } else {
        if (interp_velocity_3d(c->m, c->f, k, ll, x, y, z, ux, uy, uz)) c->err = 1;
    }
}

/* update_state_lsm1.pyx:135-177 */
static void euler_lsm1(ctx_t *c) {
    double ux, uy, uz, dt = c->p->dt;
    double z = c->pd == 3 ? POS(c, 2) : 0.;
    lsm1_velocity(c, c->s->tri[c->i], c->s->lowerlayer[c->i], POS(c, 0), POS(c, 1), z,
                  &ux, &uy, &uz);
    POS(c, 0) += ux * dt;
    POS(c, 1) += uy * dt;
    VEL(c, 0) = ux; VEL(c, 1) = uy;
    FVS(c, 0) = ux; FVS(c, 1) = uy;
    if (c->pd == 3) {
        POS(c, 2) += uz * dt;
        VEL(c, 2) = uz;
        FVS(c, 2) = uz;
    }
}

/* stage localization + early exit shared by rk2/rk3/rk4
 * (update_state_lsm1.pyx:228-248). Returns 1 when the step stops. */
static int rk_stage_locate(ctx_t *c, double xt, double yt, double zt,
                           int *tmp_tri, int *tmp_ll, int *bnd) {
    double dt = c->p->dt;
    c->s->last_tri[c->i] = c->s->tri[c->i];
    cgo_xy_localize(c->m, c->s->last_tri[c->i], LPOS(c, 0), LPOS(c, 1), xt, yt, tmp_tri, bnd);
    *tmp_ll = 0;
    if (c->pd == 3) *tmp_ll = z_localize(c->m, c->f, *tmp_tri, xt, yt, zt);
    if (*bnd != -1 || (c->pd == 3 && (*tmp_ll == -2 || *tmp_ll == -3))) {
        c->s->tri[c->i] = *tmp_tri;
        if (c->pd == 3) c->s->lowerlayer[c->i] = *tmp_ll;
        POS(c, 0) += VEL(c, 0) * dt;
        POS(c, 1) += VEL(c, 1) * dt;
        if (c->pd == 3) POS(c, 2) += VEL(c, 2) * dt;
        return 1;
    }
    /* stage point outside the mesh without a boundary crossing: the
     * reference's next interpolation raises ValueError */
    if (*tmp_tri < 0) { c->err = 1; return 1; }
    return 0;
}

static void set_up_us(ctx_t *c, double ux, double uy, double uz) {
    VEL(c, 0) = ux; VEL(c, 1) = uy;
    FVS(c, 0) = ux; FVS(c, 1) = uy;
    if (c->pd == 3) { VEL(c, 2) = uz; FVS(c, 2) = uz; }
}

/* update_state_lsm1.pyx:179-274 */
static int rk2_lsm1(ctx_t *c) {
    double ux, uy, uz, dt = c->p->dt, xt, yt, zt = 0.;
    int tt, tl, bnd;
    double z = c->pd == 3 ? POS(c, 2) : 0.;
    lsm1_velocity(c, c->s->tri[c->i], c->s->lowerlayer[c->i], POS(c, 0), POS(c, 1), z, &ux, &uy, &uz);
    set_up_us(c, ux, uy, uz);
    xt = POS(c, 0) + 0.5 * ux * dt;
    yt = POS(c, 1) + 0.5 * uy * dt;
    if (c->pd == 3) zt = POS(c, 2) + 0.5 * uz * dt;
    if (rk_stage_locate(c, xt, yt, zt, &tt, &tl, &bnd)) return bnd;
    lsm1_velocity(c, tt, tl, xt, yt, zt, &ux, &uy, &uz);
    POS(c, 0) += ux * dt;
    POS(c, 1) += uy * dt;
    if (c->pd == 3) POS(c, 2) += uz * dt;
    return -1;
}

/* update_state_lsm1.pyx:276-432 */
static int rk3_lsm1(ctx_t *c) {
    double ux, uy, uz, dt = c->p->dt, xt, yt, zt;
    double k1x, k1y, k1z = 0., k2x, k2y, k2z = 0., k3x, k3y, k3z = 0.;
    int tt, tl, bnd;
    double z = c->pd == 3 ? POS(c, 2) : 0.;
    lsm1_velocity(c, c->s->tri[c->i], c->s->lowerlayer[c->i], POS(c, 0), POS(c, 1), z, &ux, &uy, &uz);
    set_up_us(c, ux, uy, uz);
    k1x = ux * dt; k1y = uy * dt;
    if (c->pd == 3) k1z = uz * dt;
    xt = POS(c, 0) + (1. / 3.) * k1x;
    yt = POS(c, 1) + (1. / 3.) * k1y;
    zt = c->pd == 3 ? POS(c, 2) + (1. / 3.) * k1z : 0.;
    if (rk_stage_locate(c, xt, yt, zt, &tt, &tl, &bnd)) return bnd;
    lsm1_velocity(c, tt, tl, xt, yt, zt, &ux, &uy, &uz);
    k2x = ux * dt; k2y = uy * dt;
    if (c->pd == 3) k2z = uz * dt;
    xt = POS(c, 0) + (2. / 3.) * k2x;
    yt = POS(c, 1) + (2. / 3.) * k2y;
    zt = c->pd == 3 ? POS(c, 2) + (2. / 3.) * k2z : 0.;
    if (rk_stage_locate(c, xt, yt, zt, &tt, &tl, &bnd)) return bnd;
    lsm1_velocity(c, tt, tl, xt, yt, zt, &ux, &uy, &uz);
    k3x = ux * dt; k3y = uy * dt;
    if (c->pd == 3) k3z = uz * dt;
    POS(c, 0) += (0.25 * k1x + 0.75 * k3x);
    POS(c, 1) += (0.25 * k1y + 0.75 * k3y);
    if (c->pd == 3) POS(c, 2) += (0.25 * k1z + 0.75 * k3z);
    (void)k2z;
    return -1;
}

/* update_state_lsm1.pyx:434-656 */
static int rk4_lsm1(ctx_t *c) {
    double ux, uy, uz, dt = c->p->dt, xt, yt, zt;
    double k1x, k1y, k1z = 0., k2x, k2y, k2z = 0., k3x, k3y, k3z = 0., k4x, k4y, k4z = 0.;
    int tt, tl, bnd;
    double z = c->pd == 3 ? POS(c, 2) : 0.;
    lsm1_velocity(c, c->s->tri[c->i], c->s->lowerlayer[c->i], POS(c, 0), POS(c, 1), z, &ux, &uy, &uz);
    set_up_us(c, ux, uy, uz);
    k1x = ux * dt; k1y = uy * dt;
    if (c->pd == 3) k1z = uz * dt;
    xt = POS(c, 0) + 0.5 * k1x;
    yt = POS(c, 1) + 0.5 * k1y;
    zt = c->pd == 3 ? POS(c, 2) + 0.5 * k1z : 0.;
    if (rk_stage_locate(c, xt, yt, zt, &tt, &tl, &bnd)) return bnd;
    lsm1_velocity(c, tt, tl, xt, yt, zt, &ux, &uy, &uz);
    k2x = ux * dt; k2y = uy * dt;
    if (c->pd == 3) k2z = uz * dt;
    xt = POS(c, 0) + 0.5 * k2x;
    yt = POS(c, 1) + 0.5 * k2y;
    zt = c->pd == 3 ? POS(c, 2) + 0.5 * k2z : 0.;
    if (rk_stage_locate(c, xt, yt, zt, &tt, &tl, &bnd)) return bnd;
    lsm1_velocity(c, tt, tl, xt, yt, zt, &ux, &uy, &uz);
    k3x = ux * dt; k3y = uy * dt;
    if (c->pd == 3) k3z = uz * dt;
    xt = POS(c, 0) + k3x;
    yt = POS(c, 1) + k3y;
    zt = c->pd == 3 ? POS(c, 2) + k3z : 0.;
    if (rk_stage_locate(c, xt, yt, zt, &tt, &tl, &bnd)) return bnd;
    lsm1_velocity(c, tt, tl, xt, yt, zt, &ux, &uy, &uz);
    k4x = ux * dt; k4y = uy * dt;
    if (c->pd == 3) k4z = uz * dt;
    POS(c, 0) += (k1x + 2. * k2x + 2. * k3x + k4x) / 6.;
    POS(c, 1) += (k1y + 2. * k2y + 2. * k3y + k4y) / 6.;
    if (c->pd == 3) POS(c, 2) += (k1z + 2. * k2z + 2. * k3z + k4z) / 6.;
    return -1;
}

/* update_state_lsm1.pyx:658-726 */
static void diffusion_lsm1(ctx_t *c, int tri0, int ll0) {
    const cgo_params *p = c->p;
    double dt = p->dt, sqrtdt = sqrt(dt);
    double xix = 0., xiy = 0., xiz = 0.;
    double diffx = 0., diffy = 0., diffz = 0.;
    double driftx = 0., drifty = 0., driftz = 0.;
    int diffmod = p->diffusion_model;
    if (diffmod == 2 || diffmod == 3) {
        double Kp = 0., dKdx = 0., dKdy = 0., dKdz = 0., z0 = 0.;
        if (c->pd == 3) z0 = LPOS(c, 2);
        if (interp_diffusivity_gradient(c->m, c->f, tri0, ll0, LPOS(c, 0), LPOS(c, 1), z0,
                                        p->sigc, &Kp, &dKdx, &dKdy, &dKdz))
            c->err = 1;
        diffx = sqrt(2. * Kp) * sqrtdt;
        diffy = diffx;
        driftx = dKdx * dt;
        drifty = dKdy * dt;
        if (c->pd == 3) {
            if (diffmod == 2) {
                diffz = sqrt(2. * p->nuz) * sqrtdt;
            } else {
                diffz = diffx;
                driftz = dKdz * dt;
            }
        }
    } else {
        diffx = sqrt(2. * p->nux) * sqrtdt;
        diffy = diffx;
        if (c->pd == 3) diffz = sqrt(2. * p->nuz) * sqrtdt;
    }
    if (diffx != 0.) rng_pair(&c->rng, p->rng_method, &xix, &xiy);
    if (c->pd == 3 && diffz != 0.) xiz = rng_single(&c->rng, p->rng_method);
    POS(c, 0) += driftx + diffx * xix;
    POS(c, 1) += drifty + diffy * xiy;
    if (c->pd == 3) POS(c, 2) += driftz + diffz * xiz;
}

/* update_state_lsm1.pyx:30-133 */
static int update_state_lsm1(ctx_t *c) {
    const cgo_params *p = c->p;
    int bnd_j = -1, i = c->i;
    int tri0 = c->s->tri[i], ll0 = 0;
    for (int d = 0; d < c->pd; d++) { LPOS(c, d) = POS(c, d); LVEL(c, d) = VEL(c, d); }
    if (c->pd == 3) ll0 = c->s->lowerlayer[i];
    switch (p->time_scheme) {
    case 1: euler_lsm1(c); break;
    case 2: bnd_j = rk2_lsm1(c); break;
    case 3: bnd_j = rk3_lsm1(c); break;
    case 4: bnd_j = rk4_lsm1(c); break;
    default: c->err = 1; return -1;
    }
    if (p->diffusion_model != 0) diffusion_lsm1(c, tri0, ll0);
    if (c->pd == 3) {
        double wb = buoyancy_velocity(p, c->s->diameter[i], 0, p->rho0);
        POS(c, 2) += wb * p->dt;
        VEL(c, 2) += wb;
    }
    if (bnd_j == -1) {
        c->s->last_tri[i] = c->s->tri[i];
        cgo_xy_localize(c->m, c->s->last_tri[i], LPOS(c, 0), LPOS(c, 1), POS(c, 0), POS(c, 1),
                        &c->s->tri[i], &bnd_j);
        if (c->pd == 3)
            c->s->lowerlayer[i] = z_localize(c->m, c->f, c->s->tri[i], POS(c, 0), POS(c, 1), POS(c, 2));
    }
    return bnd_j;
}

/* ======================================================================
 * Fields needed by LSM2 / LSM3
 * ====================================================================== */

/* eulerian_field_set.pyx:1184-1287 with zlocalize == 0 (layer given) */
static int interp_field_3d(const cgo_mesh *m, const cgo_fields *f, const double *fld,
                           int k, int ll, double x, double y, double z, double *out) {
    p1_t p = p1_factors(m, k, x, y);
    if (ll == PART_LOC_B || ll == PART_LOC_A) return -1;
    int jl = ll * f->npoints, ju = (ll + 1) * f->npoints;
    double zlp = p1_eval(f->zs, jl, &p);
    double zup = p1_eval(f->zs, ju, &p);
    double dz = zlp - zup;
    if (fabs(dz) < EPSILON) return -2;
    double zf0 = (z - zup) / dz;
    double zf1 = (zlp - z) / dz;
    double resl = p1_eval(fld, jl, &p);
    double resu = p1_eval(fld, ju, &p);
    *out = zf0 * resl + zf1 * resu;
    return 0;
}

/* turbulent energy and dissipation at the particle, 2D P1 or 3D prism */
static int turb_fields(ctx_t *c, int k, int ll, double x, double y, double z,
                       double *kt, double *ep) {
    if (c->f->dim == 2) {
        *kt = interp_field_2d(c->m, c->f, c->f->kt, k, -1, x, y);
        *ep = interp_field_2d(c->m, c->f, c->f->ep, k, -1, x, y);
        return 0;
    }
    if (interp_field_3d(c->m, c->f, c->f->kt, k, ll, x, y, z, kt)) return -1;
    if (interp_field_3d(c->m, c->f, c->f->ep, k, ll, x, y, z, ep)) return -1;
    return 0;
}

/* eulerian_field_set.pyx:1396-1454 */
static void interp_acceleration_2d(ctx_t *c, int k, double x, double y, double dt,
                                   double ua, double va, double *ax, double *ay) {
    const cgo_mesh *m = c->m;
    const cgo_fields *f = c->f;
    const double *u = f->ux, *v = f->uy, *u0 = f->u0, *v0 = f->v0;
    const double *gx = m->gradx + 3 * k, *gy = m->grady + 3 * k;
    int i0 = m->tri[3 * k], i1 = m->tri[3 * k + 1], i2 = m->tri[3 * k + 2];
    double dudx = u[i0] * gx[0] + u[i1] * gx[1] + u[i2] * gx[2];
    double dudy = u[i0] * gy[0] + u[i1] * gy[1] + u[i2] * gy[2];
    double dvdx = v[i0] * gx[0] + v[i1] * gx[1] + v[i2] * gx[2];
    double dvdy = v[i0] * gy[0] + v[i1] * gy[1] + v[i2] * gy[2];
    double dudt = 0., dvdt = 0.;
    if (f->frozen == 0 && f->prev_valid) {
        p1_t p = p1_factors(m, k, x, y);
        dudt = ((u[i0] - u0[i0]) * p.f0 + (u[i1] - u0[i1]) * p.f1 + (u[i2] - u0[i2]) * p.f2) / dt;
        dvdt = ((v[i0] - v0[i0]) * p.f0 + (v[i1] - v0[i1]) * p.f1 + (v[i2] - v0[i2]) * p.f2) / dt;
    }
    *ax = dudt + ua * dudx + va * dudy;
    *ay = dvdt + ua * dvdx + va * dvdy;
}

/* eulerian_field_set.pyx:1999-2023 */
static void prism_value_gradient(const double *fld, int jl, int ju, const p1_t *p,
                                 const double *gx, const double *gy, double s, double dz,
                                 double zlx, double zly, double zux, double zuy,
                                 double *val, double *ddx, double *ddy, double *ddz) {
    double fl = fld[jl + p->i0] * p->f0 + fld[jl + p->i1] * p->f1 + fld[jl + p->i2] * p->f2;
    double fu = fld[ju + p->i0] * p->f0 + fld[ju + p->i1] * p->f1 + fld[ju + p->i2] * p->f2;
    double gxl = fld[jl + p->i0] * gx[0] + fld[jl + p->i1] * gx[1] + fld[jl + p->i2] * gx[2];
    double gyl = fld[jl + p->i0] * gy[0] + fld[jl + p->i1] * gy[1] + fld[jl + p->i2] * gy[2];
    double gxu = fld[ju + p->i0] * gx[0] + fld[ju + p->i1] * gx[1] + fld[ju + p->i2] * gx[2];
    double gyu = fld[ju + p->i0] * gy[0] + fld[ju + p->i1] * gy[1] + fld[ju + p->i2] * gy[2];
    double dfdz = (fu - fl) / dz;
    *val = (1. - s) * fl + s * fu;
    *ddx = (1. - s) * gxl + s * gxu - dfdz * ((1. - s) * zlx + s * zux);
    *ddy = (1. - s) * gyl + s * gyu - dfdz * ((1. - s) * zly + s * zuy);
    *ddz = dfdz;
}

/* eulerian_field_set.pyx:1456-1579 */
static int interp_acceleration_3d(ctx_t *c, int k, int ll, double x, double y, double z,
                                  double dt, double ua, double va, double wa,
                                  double *ax, double *ay, double *az) {
    const cgo_mesh *m = c->m;
    const cgo_fields *f = c->f;
    p1_t p = p1_factors(m, k, x, y);
    const double *gx = m->gradx + 3 * k, *gy = m->grady + 3 * k;
    if (ll == PART_LOC_B || ll == PART_LOC_A) return -1;
    int jl = ll * f->npoints, ju = (ll + 1) * f->npoints;
    const double *el = f->zs;
    double zlp = p1_eval(el, jl, &p);
    double zup = p1_eval(el, ju, &p);
    double dz = zup - zlp;
    if (fabs(dz) < EPSILON) return -2;
    double s = (z - zlp) / dz;
    double zlx = el[jl + p.i0] * gx[0] + el[jl + p.i1] * gx[1] + el[jl + p.i2] * gx[2];
    double zly = el[jl + p.i0] * gy[0] + el[jl + p.i1] * gy[1] + el[jl + p.i2] * gy[2];
    double zux = el[ju + p.i0] * gx[0] + el[ju + p.i1] * gx[1] + el[ju + p.i2] * gx[2];
    double zuy = el[ju + p.i0] * gy[0] + el[ju + p.i1] * gy[1] + el[ju + p.i2] * gy[2];
    double un, dudx, dudy, dudz, vn, dvdx, dvdy, dvdz, wn, dwdx, dwdy, dwdz, t0, t1, t2, t3;
    prism_value_gradient(f->ux, jl, ju, &p, gx, gy, s, dz, zlx, zly, zux, zuy, &un, &dudx, &dudy, &dudz);
    prism_value_gradient(f->uy, jl, ju, &p, gx, gy, s, dz, zlx, zly, zux, zuy, &vn, &dvdx, &dvdy, &dvdz);
    prism_value_gradient(f->uz, jl, ju, &p, gx, gy, s, dz, zlx, zly, zux, zuy, &wn, &dwdx, &dwdy, &dwdz);
    double dudt = 0., dvdt = 0., dwdt = 0.;
    if (f->frozen == 0 && f->prev_valid) {
        prism_value_gradient(f->u0, jl, ju, &p, gx, gy, s, dz, zlx, zly, zux, zuy, &t0, &t1, &t2, &t3);
        dudt = (un - t0) / dt;
        prism_value_gradient(f->v0, jl, ju, &p, gx, gy, s, dz, zlx, zly, zux, zuy, &t0, &t1, &t2, &t3);
        dvdt = (vn - t0) / dt;
        prism_value_gradient(f->w0, jl, ju, &p, gx, gy, s, dz, zlx, zly, zux, zuy, &t0, &t1, &t2, &t3);
        dwdt = (wn - t0) / dt;
    }
    *ax = dudt + ua * dudx + va * dudy + wa * dudz;
    *ay = dvdt + ua * dvdx + va * dvdy + wa * dvdz;
    *az = dwdt + ua * dwdx + va * dwdy + wa * dwdz;
    return 0;
}

/* x**y for x >= 0 as the compiled reference evaluates it: Cython (cpow
 * directive off) gives double ** double a complex result, computed by the C
 * library's cpow, i.e. exp(y * log|x|) through the complex logarithm (whose
 * real part uses log1p((x-1)(x+1))/2 for 0.5 <= x < 2).  This differs from
 * pow(x, y) in the last bits, so the restatement calls cpow too. */
static double cpow_re(double x, double y) {
    return creal(cpow(CMPLX(x, 0.), CMPLX(y, 0.)));
}

/* lagrangian_particle_set.pyx:790-832 (the powers with a non-integer or a
 * fractional-looking exponent go through cpow_re, as in the compiled
 * reference; (24/Re)**10, 0.4**10, 0.5**-10, 0.2**-10 and the last three
 * powers are real pow) */
static double drag_coefficient(const cgo_params *p, double U, double dp) {
    double Re = fmax(EPSILON, U * dp / NU0);
    if (p->drag_model == 0) return p->drag_coef;
    if (p->drag_model == 1) {
        if (Re <= 1000.) return (24. / Re) * (1. + 0.15 * cpow_re(Re, 0.687));
        return 0.44;
    }
    if (p->drag_model == 2) {
        double phi1 = pow(24. / Re, 10.) + cpow_re(21. * cpow_re(Re, -0.67), 10.) +
                      cpow_re(4. * cpow_re(Re, -0.33), 10.) + pow(0.4, 10.);
        double phi2 = 1. / (cpow_re(0.148 * cpow_re(Re, 0.11), -10.) + pow(0.5, -10.));
        double phi3 = cpow_re(1.57 * cpow_re(Re, -1.625) * 1.e8, 10.);
        double phi4 = 1. / (cpow_re(6e-17 * cpow_re(Re, 2.63), -10.) + pow(0.2, -10.));
        return pow(1. / (pow(phi1 + phi2, -1.) + pow(phi3, -1.)) + phi4, 1. / 10.);
    }
    return 0.44;
}

/* the mean velocity of the LSM2/3 schemes at (k, ll, x, y, z) */
static void mean_velocity(ctx_t *c, int k, int ll, double x, double y, double z,
                          double *ux, double *uy, double *uz) {
    lsm1_velocity(c, k, ll, x, y, z, ux, uy, uz);
}

static void mean_acceleration(ctx_t *c, int k, int ll, double x, double y, double z,
                              double ux, double uy, double uz,
                              double *ax, double *ay, double *az) {
    if (c->f->dim == 2) {
        interp_acceleration_2d(c, k, x, y, c->p->dt, ux, uy, ax, ay);
        *az = 0.;
    } else {
        if (interp_acceleration_3d(c, k, ll, x, y, z, c->p->dt, ux, uy, uz, ax, ay, az)) c->err = 1;
    }
}

/* ======================================================================
 * LSM2 (cylag/lsm/update_state_lsm2.pyx)
 * ====================================================================== */

/* drag rate a1 = A1c (1.5/dp) Cd |U - Up| for a slip (dx, dy, dz),
 * update_state_lsm2.pyx:192-198: ((a1c*(1.5/dp))*Cd)*unorm */
static double lsm2_a1(ctx_t *c, double rx, double ry, double rz) {
    double unorm = c->pd == 2 ? sqrt(rx * rx + ry * ry) : sqrt(rx * rx + ry * ry + rz * rz);
    unorm = fmax(EPSILON_LSM2, unorm);
    double dp = c->s->diameter[c->i];
    double Cd = drag_coefficient(c->p, unorm, dp);
    return c->p->a1c * (1.5 / dp) * Cd * unorm;
}

/* update_state_lsm2.pyx:141-217 */
static void euler_lsm2(ctx_t *c) {
    const cgo_params *p = c->p;
    double dt = p->dt, ux, uy, uz, ax = 0., ay = 0., az = 0.;
    double z = c->pd == 3 ? POS(c, 2) : 0.;
    int k = c->s->tri[c->i], ll = c->s->lowerlayer[c->i];
    mean_velocity(c, k, ll, POS(c, 0), POS(c, 1), z, &ux, &uy, &uz);
    if (p->added_mass) mean_acceleration(c, k, ll, POS(c, 0), POS(c, 1), z, ux, uy, uz, &ax, &ay, &az);
    double a1 = lsm2_a1(c, ux - VEL(c, 0), uy - VEL(c, 1), c->pd == 3 ? uz - VEL(c, 2) : 0.);
    FVS(c, 0) = ux;
    FVS(c, 1) = uy;
    VEL(c, 0) += (ux - VEL(c, 0)) * dt * a1 + ax * p->a2c * dt;
    VEL(c, 1) += (uy - VEL(c, 1)) * dt * a1 + ay * p->a2c * dt;
    POS(c, 0) += VEL(c, 0) * dt;
    POS(c, 1) += VEL(c, 1) * dt;
    if (c->pd == 3) {
        FVS(c, 2) = uz;
        VEL(c, 2) += (uz - VEL(c, 2)) * dt * a1 + az * p->a2c * dt - GRAV * p->a0c * dt;
        POS(c, 2) += VEL(c, 2) * dt;
    }
}

/* Runge-Kutta schemes of LSM2 (update_state_lsm2.pyx:219-1021).  Stage s
 * evaluates U (and the added-mass acceleration) at the stage point, the
 * slip against up + cs f(s-1), and k = (up + cs f(s-1)) dt,
 * f = (U - (up + cs f(s-1))) dt a1 + a a2c dt [- g a0c dt]. */
static int rk_lsm2(ctx_t *c, int scheme) {
    const cgo_params *p = c->p;
    double dt = p->dt, ux, uy, uz, ax = 0., ay = 0., az = 0.;
    int pd = c->pd, i = c->i;
    double kx[4] = {0}, ky[4] = {0}, kz[4] = {0}, fx[4] = {0}, fy[4] = {0}, fz[4] = {0};
    int nst = scheme == 2 ? 2 : (scheme == 3 ? 3 : 4);
    /* stage point offsets (applied to k) and slip offsets (applied to f) */
    double cpos[4], cvel[4];
    if (scheme == 2) { cpos[1] = 0.5; cvel[1] = 0.5; }
    else if (scheme == 3) { cpos[1] = 1. / 3.; cvel[1] = 1. / 3.; cpos[2] = 2. / 3.; cvel[2] = 2. / 3.; }
    else { cpos[1] = 0.5; cvel[1] = 0.5; cpos[2] = 0.5; cvel[2] = 0.5; cpos[3] = 1.; cvel[3] = 1.; }
    int k = c->s->tri[i], ll = c->s->lowerlayer[i];
    double xs = POS(c, 0), ys = POS(c, 1), zs = pd == 3 ? POS(c, 2) : 0.;
    for (int st = 0; st < nst; st++) {
        mean_velocity(c, k, ll, xs, ys, zs, &ux, &uy, &uz);
        if (p->added_mass) mean_acceleration(c, k, ll, xs, ys, zs, ux, uy, uz, &ax, &ay, &az);
        double a1;
        double vx, vy, vz;
        if (st == 0) {
            a1 = lsm2_a1(c, ux - VEL(c, 0), uy - VEL(c, 1), pd == 3 ? uz - VEL(c, 2) : 0.);
            vx = VEL(c, 0); vy = VEL(c, 1); vz = pd == 3 ? VEL(c, 2) : 0.;
            kx[0] = vx * dt; ky[0] = vy * dt;
            fx[0] = (ux - vx) * dt * a1 + ax * p->a2c * dt;
            fy[0] = (uy - vy) * dt * a1 + ay * p->a2c * dt;
            if (pd == 3) {
                kz[0] = vz * dt;
                fz[0] = (uz - vz) * dt * a1 + az * p->a2c * dt - GRAV * p->a0c * dt;
            }
        } else {
            double cv = cvel[st];
            /* slip: (ux-up[0]-cv*f)**2 ... evaluated left to right */
            double sx = ux - VEL(c, 0) - cv * fx[st - 1];
            double sy = uy - VEL(c, 1) - cv * fy[st - 1];
            double sz = pd == 3 ? uz - VEL(c, 2) - cv * fz[st - 1] : 0.;
            a1 = lsm2_a1(c, sx, sy, sz);
            vx = VEL(c, 0) + cv * fx[st - 1];
            vy = VEL(c, 1) + cv * fy[st - 1];
            kx[st] = vx * dt; ky[st] = vy * dt;
            fx[st] = (ux - vx) * dt * a1 + ax * p->a2c * dt;
            fy[st] = (uy - vy) * dt * a1 + ay * p->a2c * dt;
            if (pd == 3) {
                vz = VEL(c, 2) + cv * fz[st - 1];
                kz[st] = vz * dt;
                fz[st] = (uz - vz) * dt * a1 + az * p->a2c * dt - GRAV * p->a0c * dt;
            }
        }
        if (st == nst - 1) {
            /* final update */
            FVS(c, 0) = ux; FVS(c, 1) = uy;
            if (scheme == 2) {
                VEL(c, 0) += fx[1]; VEL(c, 1) += fy[1];
                POS(c, 0) += kx[1]; POS(c, 1) += ky[1];
                if (pd == 3) { FVS(c, 2) = uz; VEL(c, 2) += fz[1]; POS(c, 2) += kz[1]; }
            } else if (scheme == 3) {
                VEL(c, 0) += (0.25 * fx[0] + 0.75 * fx[2]);
                VEL(c, 1) += (0.25 * fy[0] + 0.75 * fy[2]);
                POS(c, 0) += (0.25 * kx[0] + 0.75 * kx[2]);
                POS(c, 1) += (0.25 * ky[0] + 0.75 * ky[2]);
                if (pd == 3) {
                    FVS(c, 2) = uz;
                    VEL(c, 2) += (0.25 * fz[0] + 0.75 * fz[2]);
                    POS(c, 2) += (0.25 * kz[0] + 0.75 * kz[2]);
                }
            } else {
                VEL(c, 0) += (1. / 6.) * (fx[0] + 2. * fx[1] + 2. * fx[2] + fx[3]);
                VEL(c, 1) += (1. / 6.) * (fy[0] + 2. * fy[1] + 2. * fy[2] + fy[3]);
                POS(c, 0) += (1. / 6.) * (kx[0] + 2. * kx[1] + 2. * kx[2] + kx[3]);
                POS(c, 1) += (1. / 6.) * (ky[0] + 2. * ky[1] + 2. * ky[2] + ky[3]);
                if (pd == 3) {
                    FVS(c, 2) = uz;
                    VEL(c, 2) += (1. / 6.) * (fz[0] + 2. * fz[1] + 2. * fz[2] + fz[3]);
                    POS(c, 2) += (1. / 6.) * (kz[0] + 2. * kz[1] + 2. * kz[2] + kz[3]);
                }
            }
            return -1;
        }
        /* next stage point and its localization (e.g. 2*, 3*, 4* stages) */
        double cp = cpos[st + 1];
        double xt = POS(c, 0) + cp * kx[st], yt = POS(c, 1) + cp * ky[st];
        double zt = pd == 3 ? POS(c, 2) + cp * kz[st] : 0.;
        int tt, tl = 0, bnd;
        c->s->last_tri[i] = c->s->tri[i];
        cgo_xy_localize(c->m, c->s->last_tri[i], LPOS(c, 0), LPOS(c, 1), xt, yt, &tt, &bnd);
        if (pd == 3) tl = z_localize(c->m, c->f, tt, xt, yt, zt);
        if (bnd != -1 || (pd == 3 && (tl == -2 || tl == -3))) {
            /* Euler step with the first-stage quantities of this stage's
             * evaluation point (update_state_lsm2.pyx:315-333) */
            c->s->tri[i] = tt;
            if (pd == 3) c->s->lowerlayer[i] = tl;
            /* note: U, a, a1 here are those of the stage just evaluated */
            FVS(c, 0) = ux; FVS(c, 1) = uy;
            VEL(c, 0) += (ux - VEL(c, 0)) * dt * a1 + ax * p->a2c * dt;
            VEL(c, 1) += (uy - VEL(c, 1)) * dt * a1 + ay * p->a2c * dt;
            if (pd == 3) {
                FVS(c, 2) = uz;
                VEL(c, 2) += (uz - VEL(c, 2)) * dt * a1 + az * p->a2c * dt - GRAV * p->a0c * dt;
            }
            POS(c, 0) += VEL(c, 0) * dt;
            POS(c, 1) += VEL(c, 1) * dt;
            if (pd == 3) POS(c, 2) += VEL(c, 2) * dt;
            return bnd;
        }
        /* outside without a boundary crossing: the reference raises
         * ValueError at the next interpolation */
        if (tt < 0) { c->err = 1; return -1; }
        k = tt; ll = tl; xs = xt; ys = yt; zs = zt;
    }
    return -1;
}

/* update_state_lsm2.pyx:1023-1086 (same law as diffusion_lsm1) */
static void diffusion_lsm2(ctx_t *c, int tri0, int ll0) { diffusion_lsm1(c, tri0, ll0); }

/* update_state_lsm2.pyx:1088-1230 */
static void euler_maruyama_lsm2_u(ctx_t *c) {
    const cgo_params *p = c->p;
    double dt = p->dt, sqrtdt = sqrt(dt), ux, uy, uz, ax = 0., ay = 0., az = 0.;
    int pd = c->pd, diffmod = p->diffusion_model, nuopt = p->diffusion_lsm2_option;
    double z = pd == 3 ? POS(c, 2) : 0.;
    int k = c->s->tri[c->i], ll = c->s->lowerlayer[c->i];
    mean_velocity(c, k, ll, POS(c, 0), POS(c, 1), z, &ux, &uy, &uz);
    if (p->added_mass) mean_acceleration(c, k, ll, POS(c, 0), POS(c, 1), z, ux, uy, uz, &ax, &ay, &az);
    double a1 = lsm2_a1(c, ux - VEL(c, 0), uy - VEL(c, 1), pd == 3 ? uz - VEL(c, 2) : 0.);
    double xix = 0., xiy = 0., xiz = 0., diffx = 0., diffy = 0., diffz = 0.;
    if (diffmod != 0) {
        rng_pair(&c->rng, p->rng_method, &xix, &xiy);
        if (pd == 3) xiz = rng_single(&c->rng, p->rng_method);
    }
    if (diffmod == 2 || diffmod == 3) {
        double kt, ep;
        if (turb_fields(c, k, ll, POS(c, 0), POS(c, 1), z, &kt, &ep)) c->err = 1;
        ep = fmax(ep, EPSILON);
        double tml = (kt / ep) / (0.5 + (3. / 4.) * C0KOLM);
        diffx = a1 * tml * sqrt(C0KOLM * ep) * sqrtdt;
        diffy = diffx;
        if (pd == 3) {
            if (diffmod == 2) diffz = nuopt == 2 ? p->nuz * sqrtdt : a1 * sqrt(2. * p->nuz) * sqrtdt;
            else diffz = diffx;
        }
    } else {
        if (nuopt == 2) {
            diffx = p->nux * sqrtdt; diffy = diffx;
            if (pd == 3) diffz = p->nuz * sqrtdt;
        } else if (nuopt == 3) {
            diffx = a1 * sqrt(2. * p->nux) * sqrtdt; diffy = diffx;
            if (pd == 3) diffz = a1 * sqrt(2. * p->nuz) * sqrtdt;
        }
    }
    FVS(c, 0) = ux;
    FVS(c, 1) = uy;
    VEL(c, 0) += (ux - VEL(c, 0)) * dt * a1 + ax * p->a2c * dt + diffx * xix;
    VEL(c, 1) += (uy - VEL(c, 1)) * dt * a1 + ay * p->a2c * dt + diffy * xiy;
    POS(c, 0) += VEL(c, 0) * dt;
    POS(c, 1) += VEL(c, 1) * dt;
    if (pd == 3) {
        FVS(c, 2) = uz;
        VEL(c, 2) += (uz - VEL(c, 2)) * dt * a1 + az * p->a2c * dt - GRAV * p->a0c * dt + diffz * xiz;
        POS(c, 2) += VEL(c, 2) * dt;
    }
}

/* update_state_lsm2.pyx:1240-1327 */
static int lsm2_direct_coefficients(double a1, double dt, double *beta, double *D1,
                                    double *D2, double *force_x, double *q_uu,
                                    double *q_xu, double *q_xx) {
    double r = a1 * dt;
    if (!isfinite(a1) || !isfinite(dt) || a1 < 0. || dt < 0. || !isfinite(r)) return -1;
    *beta = exp(-r);
    if (r < 0.1) {
        double phi1 = 1., phi2 = 0.5, term = 1.;
        for (int n = 1; n < 13; n++) {
            term *= -r / (n + 1.);
            phi1 += term;
            phi2 += term / (n + 2.);
        }
        *D1 = dt * phi1;
        *D2 = dt * r * phi2;
        *force_x = dt * dt * phi2;
    } else {
        *D1 = -expm1(-r) / a1;
        *D2 = dt - *D1;
        *force_x = *D2 / a1;
    }
    if (r == 0.) *q_uu = dt;
    else *q_uu = dt * (-expm1(-2. * r) / (2. * r));
    *q_xu = 0.5 * *D1 * *D1;
    if (r < 1.) {
        double term = 1. / 6., power2 = 4., qxx = 1. / 3.;
        for (int n = 1; n < 24; n++) {
            term *= -r / (n + 3.);
            power2 *= 2.;
            qxx += (power2 - 2.) * term;
        }
        *q_xx = qxx * dt * dt * dt;
    } else {
        *q_xx = ((dt - 2. * *D1 + *q_uu) / a1) / a1;
    }
    return 0;
}

/* update_state_lsm2.pyx:1329-1542 (diffmod 0: di_ode_lsm2, 1232-1238) */
static void di_lsm2(ctx_t *c, int diffmod, double nux, double nuz, int nuopt) {
    const cgo_params *p = c->p;
    double dt = p->dt, ux, uy, uz, ax = 0., ay = 0., az = 0.;
    int pd = c->pd;
    double xp0[3], up0[3];
    for (int d = 0; d < pd; d++) { xp0[d] = POS(c, d); up0[d] = VEL(c, d); }
    int k = c->s->tri[c->i], ll = c->s->lowerlayer[c->i];
    double z0 = pd == 3 ? xp0[2] : 0.;
    mean_velocity(c, k, ll, xp0[0], xp0[1], z0, &ux, &uy, &uz);
    if (p->added_mass) mean_acceleration(c, k, ll, xp0[0], xp0[1], z0, ux, uy, uz, &ax, &ay, &az);
    double unorm;
    if (pd == 2) unorm = sqrt((ux - up0[0]) * (ux - up0[0]) + (uy - up0[1]) * (uy - up0[1]));
    else unorm = sqrt((ux - up0[0]) * (ux - up0[0]) + (uy - up0[1]) * (uy - up0[1]) +
                      (uz - up0[2]) * (uz - up0[2]));
    unorm = fmax(EPSILON_LSM2, unorm);
    double dp = c->s->diameter[c->i];
    double Cd = drag_coefficient(p, unorm, dp);
    double a1 = p->a1c * (1.5 / dp) * Cd * unorm;
    double beta, D1, D2, force_x, q_uu, q_xu, q_xx;
    if (lsm2_direct_coefficients(a1, dt, &beta, &D1, &D2, &force_x, &q_uu, &q_xu, &q_xx)) {
        c->err = 1;
        return;
    }
    double um_beta = -expm1(-a1 * dt);
    double b2[3] = {0., 0., 0.};
    if (diffmod == 2 || diffmod == 3) {
        double kt, ep;
        if (turb_fields(c, k, ll, xp0[0], xp0[1], z0, &kt, &ep)) c->err = 1;
        ep = fmax(ep, EPSILON);
        double tml = (kt / ep) / (0.5 + (3. / 4.) * C0KOLM);
        b2[0] = a1 * a1 * C0KOLM * ep * (tml * tml);
        b2[1] = b2[0];
        if (diffmod == 2) b2[2] = nuopt == 2 ? nuz * nuz : 2. * nuz * a1 * a1;
        else b2[2] = b2[0];
    } else if (diffmod != 0) {
        if (nuopt == 2) { b2[0] = nux * nux; b2[1] = b2[0]; b2[2] = nuz * nuz; }
        else if (nuopt == 3) { b2[0] = 2. * nux * a1 * a1; b2[1] = b2[0]; b2[2] = 2. * nuz * a1 * a1; }
    }
    for (int d = 0; d < pd; d++) {
        double u_k = d == 0 ? ux : (d == 1 ? uy : uz);
        double Fp = d == 0 ? p->a2c * ax : (d == 1 ? p->a2c * ay : p->a2c * az - GRAV * p->a0c);
        double up_mean = up0[d] * beta + u_k * um_beta + Fp * D1;
        double xp_mean = xp0[d] + up0[d] * D1 + u_k * D2 + Fp * force_x;
        if (b2[d] == 0. || dt == 0.) {
            FVS(c, d) = u_k;
            VEL(c, d) = up_mean;
            POS(c, d) = xp_mean;
            continue;
        }
        double var_gp = b2[d] * q_uu, cov = b2[d] * q_xu, var_gx = b2[d] * q_xx;
        double L_pp = sqrt(fmax(0., var_gp));
        double L_xp = L_pp > 0. ? cov / L_pp : 0.;
        double L_xx = sqrt(fmax(0., var_gx - L_xp * L_xp));
        double xix, xiy;
        rng_pair(&c->rng, p->rng_method, &xix, &xiy);
        double Gp = L_pp * xix;
        double Gx = L_xp * xix + L_xx * xiy;
        FVS(c, d) = u_k;
        VEL(c, d) = up_mean + Gp;
        POS(c, d) = xp_mean + Gx;
    }
}

/* update_state_lsm2.pyx:30-139 */
static int update_state_lsm2(ctx_t *c) {
    const cgo_params *p = c->p;
    int bnd_j = -1, i = c->i, diffmod = p->diffusion_model, nuopt = p->diffusion_lsm2_option;
    int tri0 = c->s->tri[i], ll0 = 0;
    for (int d = 0; d < c->pd; d++) { LPOS(c, d) = POS(c, d); LVEL(c, d) = VEL(c, d); }
    if (c->pd == 3) ll0 = c->s->lowerlayer[i];
    if (nuopt == 1 || (nuopt >= 2 && diffmod == 0)) {
        switch (p->time_scheme) {
        case 1: euler_lsm2(c); break;
        case 2: case 3: case 4: bnd_j = rk_lsm2(c, p->time_scheme); break;
        case 5: di_lsm2(c, 0, 0., 0., 2); break;
        default: c->err = 1; return -1;
        }
        if (diffmod != 0) diffusion_lsm2(c, tri0, ll0);
    } else {
        if (p->time_scheme == 1) euler_maruyama_lsm2_u(c);
        else if (p->time_scheme == 5) di_lsm2(c, diffmod, p->nux, p->nuz, nuopt);
        else { c->err = 1; return -1; }
    }
    (void)bnd_j;
    /* localization is unconditional (update_state_lsm2.pyx:122-137) */
    c->s->last_tri[i] = c->s->tri[i];
    cgo_xy_localize(c->m, c->s->last_tri[i], LPOS(c, 0), LPOS(c, 1), POS(c, 0), POS(c, 1),
                    &c->s->tri[i], &bnd_j);
    if (c->pd == 3)
        c->s->lowerlayer[i] = z_localize(c->m, c->f, c->s->tri[i], POS(c, 0), POS(c, 1), POS(c, 2));
    return bnd_j;
}

/* init_lsm2_fluctuations.pyx:28-129 */
static int lsm2_fluctuations(ctx_t *c, double *f1, double *f2, double *f3) {
    const cgo_params *p = c->p;
    *f1 = *f2 = *f3 = 0.;
    if (p->diffusion_model == 0) return 0;
    double unorm = EPSILON_LSM2, dp = c->s->diameter[c->i];
    double Cd = drag_coefficient(p, unorm, dp);
    double a1 = p->a1c * (1.5 / dp) * Cd * unorm;
    if (a1 == 0.) {
        if (p->diffusion_lsm2_option == 2 &&
            ((p->diffusion_model != 2 && p->diffusion_model != 3 && p->nux != 0.) ||
             (c->pd == 3 && p->diffusion_model != 3 && p->nuz != 0.)))
            return -1;
        return 0;
    }
    double b0, b1, b2;
    if (p->diffusion_model == 2 || p->diffusion_model == 3) {
        double kt, ep, z = c->pd == 3 ? POS(c, 2) : 0.;
        if (turb_fields(c, c->s->tri[c->i], c->s->lowerlayer[c->i], POS(c, 0), POS(c, 1), z, &kt, &ep))
            c->err = 1;
        ep = fmax(ep, EPSILON);
        double tml = (kt / ep) / (0.5 + (3. / 4.) * C0KOLM);
        b0 = a1 * C0KOLM * ep * (tml * tml);
        b1 = b0;
        if (p->diffusion_model == 2)
            b2 = p->diffusion_lsm2_option == 2 ? (p->nuz * p->nuz) / a1 : 2. * p->nuz * a1;
        else b2 = b0;
    } else {
        if (p->diffusion_lsm2_option == 2) {
            b0 = (p->nux * p->nux) / a1; b1 = b0; b2 = (p->nuz * p->nuz) / a1;
        } else {
            b0 = 2. * p->nux * a1; b1 = b0; b2 = 2. * p->nuz * a1;
        }
    }
    if (b0 > 0.) {
        double xix, xiy;
        rng_pair(&c->rng, p->rng_method, &xix, &xiy);
        *f1 = sqrt(0.5 * b0) * xix;
        *f2 = sqrt(0.5 * b1) * xiy;
    }
    if (c->pd == 3 && b2 > 0.) *f3 = sqrt(0.5 * b2) * rng_single(&c->rng, p->rng_method);
    return 0;
}

/* ======================================================================
 * LSM3 (cylag/lsm/update_state_lsm3.pyx)
 * ====================================================================== */

/* update_state_lsm3.pyx:32-216 (lsm3_edge_opt = 1) */
static int lsm3_direct_coefficients(double a, double a2, double tl, double dt, double *phi,
                                    double *q, double *force, double *flow) {
    if (!isfinite(a) || !isfinite(a2) || !isfinite(tl) || !isfinite(dt) || a < 0. || tl <= 0. || dt < 0.)
        return -1;
    double b = 1. / tl;
    if (!isfinite(b) || !isfinite(a * dt) || !isfinite(b * dt) || !isfinite(a * (1. - a2) * dt)) return -1;
    for (int k = 0; k < 9; k++) { phi[k] = 0.; q[k] = 0.; }
    phi[0] = phi[4] = phi[8] = 1.;
    for (int k = 0; k < 3; k++) { force[k] = 0.; flow[k] = 0.; }
    if (dt == 0.) return 0;
    double h = dt;
    int doublings = 0;
    while (h > 0. && fmax(a * h, b * h) > 0.5) { h *= 0.5; doublings += 1; }
    double ah = a * h, bh = b * h, kh = a * (1. - a2) * h;
    double qbar[10];
    qbar[0] = 1.;
    for (int k = 1; k < 10; k++) qbar[k] = 0.;
    double tss = 1., tsp = 0., tsx = 0., tpp = 0., tpx = 0., txx = 0.;
    double tsi = 0., tpi = 0., txi = 0., tii = 0.;
    double s = 1., pp = 0., x = 0., si = 0.;
    double sum_p = 0., sum_x = 0., sum_si = 0., int_p = 0., int_x = 0., int_si = 0.;
    double beta_term = 1., phi1 = 1., phi2 = 0.5;
    for (int n = 1; n < 25; n++) {
        double divisor = n + 1.;
        double nss = -2. * bh * tss / divisor;
        double nsp = (tss - (ah + bh) * tsp) / divisor;
        double nsx = (tsp - bh * tsx) / divisor;
        double npp = (2. * tsp - 2. * ah * tpp) / divisor;
        double npx = (tsx + tpp - ah * tpx) / divisor;
        double nxx = 2. * tpx / divisor;
        double nsi = (tss - bh * tsi) / divisor;
        double npi = (tsi + tsp - ah * tpi) / divisor;
        double nxi = (tpi + tsx) / divisor;
        double nii = 2. * tsi / divisor;
        tss = nss; tsp = nsp; tsx = nsx;
        tpp = npp; tpx = npx; txx = nxx;
        tsi = nsi; tpi = npi; txi = nxi; tii = nii;
        qbar[0] += tss; qbar[1] += tsp; qbar[2] += tsx; qbar[3] += tpp; qbar[4] += tpx;
        qbar[5] += txx; qbar[6] += tsi; qbar[7] += tpi; qbar[8] += txi; qbar[9] += tii;
        double sn = -bh * s / n, pn = (s - ah * pp) / n, xn = pp / n, sin_ = s / n;
        s = sn; pp = pn; x = xn; si = sin_;
        sum_p += pp; sum_x += x; sum_si += si;
        int_p += pp / (n + 1.); int_x += x / (n + 1.); int_si += si / (n + 1.);
        beta_term *= -ah / n;
        phi1 += beta_term / (n + 1.);
        phi2 += beta_term / ((n + 1.) * (n + 2.));
    }
    q[0] = h * qbar[0];
    q[1] = q[3] = h * kh * qbar[1];
    q[2] = q[6] = h * h * (kh * qbar[2] + a2 * qbar[6]);
    q[4] = h * kh * kh * qbar[3];
    q[5] = q[7] = h * h * kh * (kh * qbar[4] + a2 * qbar[7]);
    q[8] = h * h * h * (kh * kh * qbar[5] + 2. * kh * a2 * qbar[8] + a2 * a2 * qbar[9]);
    phi[0] = exp(-bh);
    phi[3] = kh * sum_p;
    phi[4] = exp(-ah);
    phi[6] = h * (kh * sum_x + a2 * sum_si);
    phi[7] = h * phi1;
    force[1] = phi[7];
    force[2] = h * h * phi2;
    flow[0] = -expm1(-bh);
    flow[1] = kh * bh * int_p;
    flow[2] = h * bh * (kh * int_x + a2 * int_si);
    for (int n = 0; n < doublings; n++) {
        double work[9], qnew[9];
        for (int r = 0; r < 3; r++)
            for (int cc = 0; cc < 3; cc++) {
                double value = 0.;
                for (int k = 0; k < r + 1; k++) value += phi[3 * r + k] * q[3 * k + cc];
                work[3 * r + cc] = value;
            }
        for (int r = 0; r < 3; r++)
            for (int cc = 0; cc < r + 1; cc++) {
                double value = q[3 * r + cc];
                for (int k = 0; k < cc + 1; k++) value += work[3 * r + k] * phi[3 * cc + k];
                qnew[3 * r + cc] = qnew[3 * cc + r] = value;
            }
        for (int k = 0; k < 9; k++) q[k] = qnew[k];
        flow[2] = 2. * flow[2] + phi[6] * flow[0] + phi[7] * flow[1];
        flow[1] = (1. + phi[4]) * flow[1] + phi[3] * flow[0];
        flow[0] = -expm1(-2. * b * h);
        phi[6] = phi[6] * (1. + phi[0]) + phi[7] * phi[3];
        phi[3] *= phi[0] + phi[4];
        force[2] = 2. * force[2] + phi[7] * phi[7];
        phi[7] *= 1. + phi[4];
        force[1] = phi[7];
        h *= 2.;
        phi[0] = exp(-b * h);
        phi[4] = exp(-a * h);
    }
    for (int k = 0; k < 9; k++) if (!isfinite(phi[k]) || !isfinite(q[k])) return -1;
    if (!isfinite(force[1]) || !isfinite(force[2])) return -1;
    for (int k = 0; k < 3; k++) if (!isfinite(flow[k])) return -1;
    return 0;
}

/* update_state_lsm3.pyx:218-233 */
static double phi1_(double z) { return z == 0. ? 1. : expm1(z) / z; }
static double exp_divdiff(double x, double y) { return exp(-fmin(x, y)) * phi1_(-fabs(x - y)); }
static double phi2_(double z) {
    if (fabs(z) < 0.05)
        return 0.5 + z * (1. / 6. + z * (1. / 24. + z * (1. / 120. + z * (1. / 720. +
               z * (1. / 5040. + z * (1. / 40320. + z / 362880.))))));
    return (expm1(z) - z) / (z * z);
}

/* update_state_lsm3.pyx:235-264 */
static void lsm3_closed_covariance(double a, double b, double a2, double h, double *q) {
    double d = a - b;
    double cc = a * (1. - a2) / d;
    double bb = (1. - a2) / d;
    double aa = (a2 + cc) / b;
    double sb = h * phi1_(-b * h), sa = h * phi1_(-a * h);
    double s2b = h * phi1_(-2. * b * h), s2a = h * phi1_(-2. * a * h);
    double sab = h * phi1_(-(a + b) * h);
    q[0] = s2b;
    q[1] = q[3] = cc * (s2b - sab);
    q[2] = q[6] = aa * (sb - s2b) - bb * (sb - sab);
    q[4] = cc * cc * (s2b - 2. * sab + s2a);
    q[5] = q[7] = cc * (aa * (sb - s2b - sa + sab) - bb * (sb - sab - sa + s2a));
    q[8] = (aa * aa * (h - 2. * sb + s2b) - 2. * aa * bb * (h - sb - sa + sab) +
            bb * bb * (h - 2. * sa + s2a));
}

/* update_state_lsm3.pyx:266-307 */
static void lsm3_clipped_covariance(double a, double b, double a2, double h, double *q) {
    double d = a - b, m = 0.5 * (a + b), x = m * h, delta;
    if (x > 1.) delta = fmin(0.5, LSM3_CLIP_STEP * sqrt(x)) / h;
    else delta = fmin(0.5, LSM3_CLIP_STEP / sqrt(x)) * m;
    if (fabs(d) >= delta) {
        lsm3_closed_covariance(a, b, a2, h, q);
    } else {
        double qp[9], qm[9];
        lsm3_closed_covariance(m + 0.5 * delta, m - 0.5 * delta, a2, h, qp);
        lsm3_closed_covariance(m - 0.5 * delta, m + 0.5 * delta, a2, h, qm);
        double w = 0.5 * (1. + d / delta);
        for (int k = 0; k < 9; k++) q[k] = qm[k] + w * (qp[k] - qm[k]);
    }
    for (int k = 0; k < 3; k++) q[4 * k] = fmax(q[4 * k], 0.);
    for (int r = 0; r < 3; r++)
        for (int cc = 0; cc < r; cc++) {
            double bound = sqrt(q[4 * r] * q[4 * cc]);
            q[3 * r + cc] = q[3 * cc + r] = fmax(-bound, fmin(bound, q[3 * r + cc]));
        }
}

/* update_state_lsm3.pyx:309-374 (lsm3_edge_opt = 2, the default) */
static int lsm3_clipped_coefficients(double a, double a2, double tl, double dt, double *phi,
                                     double *q, double *force, double *flow) {
    if (!isfinite(a) || !isfinite(a2) || !isfinite(tl) || !isfinite(dt) || a < 0. || tl <= 0. || dt < 0.)
        return -1;
    double b = 1. / tl;
    if (!isfinite(b) || !isfinite(a * dt) || !isfinite(b * dt) || !isfinite(a * (1. - a2) * dt)) return -1;
    for (int j = 0; j < 9; j++) { phi[j] = 0.; q[j] = 0.; }
    phi[0] = phi[4] = phi[8] = 1.;
    for (int j = 0; j < 3; j++) { force[j] = 0.; flow[j] = 0.; }
    if (dt == 0.) return 0;
    double ah = a * dt, bh = b * dt, k = a * (1. - a2);
    double alpha = exp(-bh), beta = exp(-ah);
    double divdiff = exp_divdiff(ah, bh);
    double ib = dt * phi1_(-bh), ia = dt * phi1_(-ah);
    phi[0] = alpha;
    phi[3] = k * dt * divdiff;
    phi[4] = beta;
    phi[6] = ib - (1. - a2) * dt * divdiff;
    phi[7] = ia;
    force[1] = ia;
    force[2] = dt * dt * phi2_(-ah);
    flow[0] = -expm1(-bh);
    flow[1] = k * dt * (phi1_(-ah) - divdiff);
    flow[2] = (a2 * (dt - ib) + (1. - a2) * (dt - ia - ib + dt * divdiff));
    lsm3_clipped_covariance(a, b, a2, dt, q);
    for (int j = 0; j < 9; j++) if (!isfinite(phi[j]) || !isfinite(q[j])) return -1;
    if (!isfinite(force[1]) || !isfinite(force[2])) return -1;
    for (int j = 0; j < 3; j++) if (!isfinite(flow[j])) return -1;
    return 0;
}

static int lsm3_coefficients(double a, double a2, double tl, double dt, int edge_opt,
                             double *phi, double *q, double *force, double *flow) {
    if (edge_opt == 2) return lsm3_clipped_coefficients(a, a2, tl, dt, phi, q, force, flow);
    return lsm3_direct_coefficients(a, a2, tl, dt, phi, q, force, flow);
}

/* update_state_lsm3.pyx:523-557 */
static int lsm3_cholesky(const double *q, double *lower) {
    for (int k = 0; k < 9; k++) lower[k] = 0.;
    for (int r = 0; r < 3; r++) {
        double pivot = q[3 * r + r];
        for (int cc = 0; cc < r; cc++) {
            double residual = q[3 * r + cc];
            for (int k = 0; k < cc; k++) residual -= lower[3 * r + k] * lower[3 * cc + k];
            if (lower[3 * cc + cc] > 0.) {
                lower[3 * r + cc] = residual / lower[3 * cc + cc];
            } else {
                double tol = (128. * DBL_EPS * sqrt(fabs(q[3 * r + r])) * sqrt(fabs(q[3 * cc + cc])));
                if (fabs(residual) > tol) return -1;
            }
            pivot -= lower[3 * r + cc] * lower[3 * r + cc];
        }
        if (pivot < 0.) {
            if (-pivot > 128. * DBL_EPS * fabs(q[3 * r + r])) return -1;
            pivot = 0.;
        }
        lower[3 * r + r] = sqrt(pivot);
    }
    return 0;
}

/* update_state_lsm3.pyx:559-585 */
static void lsm3_cholesky_clipped(const double *q, double *lower) {
    for (int k = 0; k < 9; k++) lower[k] = 0.;
    for (int r = 0; r < 3; r++) {
        double remaining = fmax(q[3 * r + r], 0.);
        for (int cc = 0; cc < r; cc++) {
            if (lower[3 * cc + cc] > 0.) {
                double value = q[3 * r + cc];
                for (int k = 0; k < cc; k++) value -= lower[3 * r + k] * lower[3 * cc + k];
                value /= lower[3 * cc + cc];
                if (value * value > remaining) value = copysign(sqrt(remaining), value);
                lower[3 * r + cc] = value;
                remaining -= value * value;
            }
        }
        lower[3 * r + r] = sqrt(fmax(remaining, 0.));
    }
}

/* slip drag rate of LSM3: ((a1c*(1.5/dp))*unorm)*Cd (update_state_lsm3.pyx:728) */
static double lsm3_a1(ctx_t *c, double unorm) {
    double dp = c->s->diameter[c->i];
    double Cd = drag_coefficient(c->p, unorm, dp);
    return c->p->a1c * (1.5 / dp) * unorm * Cd;
}

/* update_state_lsm3.pyx:664-820 */
static void euler_maruyama_lsm3(ctx_t *c) {
    const cgo_params *p = c->p;
    double dt = p->dt, sqrtdt = sqrt(dt), ux, uy, uz, ax = 0., ay = 0., az = 0.;
    int pd = c->pd, diffmod = p->diffusion_model;
    double z = pd == 3 ? POS(c, 2) : 0.;
    int k = c->s->tri[c->i], ll = c->s->lowerlayer[c->i];
    mean_velocity(c, k, ll, POS(c, 0), POS(c, 1), z, &ux, &uy, &uz);
    mean_acceleration(c, k, ll, POS(c, 0), POS(c, 1), z, ux, uy, uz, &ax, &ay, &az);
    double unorm;
    if (pd == 2) unorm = sqrt((FVS(c, 0) - VEL(c, 0)) * (FVS(c, 0) - VEL(c, 0)) +
                              (FVS(c, 1) - VEL(c, 1)) * (FVS(c, 1) - VEL(c, 1)));
    else unorm = sqrt((FVS(c, 0) - VEL(c, 0)) * (FVS(c, 0) - VEL(c, 0)) +
                      (FVS(c, 1) - VEL(c, 1)) * (FVS(c, 1) - VEL(c, 1)) +
                      (FVS(c, 2) - VEL(c, 2)) * (FVS(c, 2) - VEL(c, 2)));
    unorm = fmax(EPSILON_LSM2, unorm);
    double a1 = lsm3_a1(c, unorm);
    double xix, xiy, xiz = 0.;
    rng_pair(&c->rng, p->rng_method, &xix, &xiy);
    if (pd == 3) xiz = rng_single(&c->rng, p->rng_method);
    double kt = 0., ep = 0., tml, unstml, diffx, diffz = 0.;
    if (diffmod == 2 || diffmod == 3) {
        if (turb_fields(c, k, ll, POS(c, 0), POS(c, 1), z, &kt, &ep)) c->err = 1;
        ep = fmax(ep, EPSILON);
    }
    if (diffmod == 2 || diffmod == 3) {
        tml = (kt / ep) / (0.5 + (3. / 4.) * C0KOLM);
        unstml = 1. / fmax(EPSILON_LSM3, tml);
        diffx = sqrt(C0KOLM * ep) * sqrtdt;
    } else {
        unstml = 1. / p->tl_h;
        diffx = sqrt(2. * p->nux) * sqrtdt / p->tl_h;
    }
    double diffy = diffx;
    double dusx = (ax + (ux - FVS(c, 0)) * unstml) * dt + diffx * xix;
    double dusy = (ay + (uy - FVS(c, 1)) * unstml) * dt + diffy * xiy;
    VEL(c, 0) += (FVS(c, 0) - VEL(c, 0)) * dt * a1;
    VEL(c, 1) += (FVS(c, 1) - VEL(c, 1)) * dt * a1;
    FVS(c, 0) += dusx;
    FVS(c, 1) += dusy;
    if (p->added_mass) { VEL(c, 0) += p->a2c * dusx; VEL(c, 1) += p->a2c * dusy; }
    POS(c, 0) += VEL(c, 0) * dt;
    POS(c, 1) += VEL(c, 1) * dt;
    if (pd == 3) {
        if (diffmod == 1 || diffmod == 2) {
            unstml = 1. / p->tl_v;
            diffz = sqrt(2. * p->nuz) * sqrtdt / p->tl_v;
        } else {
            tml = (kt / ep) / (0.5 + (3. / 4.) * C0KOLM);
            unstml = 1. / fmax(EPSILON_LSM3, tml);
            diffz = sqrt(C0KOLM * ep) * sqrtdt;
        }
        double dusz = (az + (uz - FVS(c, 2)) * unstml) * dt + diffz * xiz;
        VEL(c, 2) += (FVS(c, 2) - VEL(c, 2)) * dt * a1 - GRAV * p->a0c * dt;
        FVS(c, 2) += dusz;
        if (p->added_mass) VEL(c, 2) += p->a2c * dusz;
        POS(c, 2) += VEL(c, 2) * dt;
    }
}

/* update_state_lsm3.pyx:822-996 */
static void di_lsm3(ctx_t *c) {
    const cgo_params *p = c->p;
    double dt = p->dt;
    if (dt == 0.) return;
    int pd = c->pd, diffmod = p->diffusion_model, edge_opt = p->lsm3_edge_opt;
    double xp0[3], up0[3], us0[3];
    for (int d = 0; d < pd; d++) { xp0[d] = POS(c, d); up0[d] = VEL(c, d); us0[d] = FVS(c, d); }
    int k = c->s->tri[c->i], ll = c->s->lowerlayer[c->i];
    double z0 = pd == 3 ? xp0[2] : 0.;
    double ux, uy, uz, ax, ay, az, kt = 0., ep = 0.;
    mean_velocity(c, k, ll, xp0[0], xp0[1], z0, &ux, &uy, &uz);
    mean_acceleration(c, k, ll, xp0[0], xp0[1], z0, ux, uy, uz, &ax, &ay, &az);
    if (diffmod == 2 || diffmod == 3)
        if (turb_fields(c, k, ll, xp0[0], xp0[1], z0, &kt, &ep)) c->err = 1;
    double unorm = (us0[0] - up0[0]) * (us0[0] - up0[0]) + (us0[1] - up0[1]) * (us0[1] - up0[1]);
    if (pd == 3) unorm += (us0[2] - up0[2]) * (us0[2] - up0[2]);
    unorm = fmax(EPSILON_LSM2, sqrt(unorm));
    double a1 = lsm3_a1(c, unorm);
    double a2 = p->added_mass ? p->a2c : 0.;
    double tl_h = p->tl_h, tl_v = p->tl_v, sigma_h, sigma_v = 0.;
    if (diffmod == 2 || diffmod == 3) {
        ep = fmax(ep, EPSILON);
        tl_h = fmax(EPSILON_LSM3, (kt / ep) / (0.5 + (3. / 4.) * C0KOLM));
        sigma_h = sqrt(C0KOLM * ep);
    } else {
        sigma_h = sqrt(2. * p->nux) / tl_h;
    }
    if (pd == 3) {
        if (diffmod == 3) { tl_v = tl_h; sigma_v = sigma_h; }
        else sigma_v = sqrt(2. * p->nuz) / tl_v;
    }
    double mean_flow[3] = {ux, uy, uz}, mean_acc[3] = {ax, ay, az};
    double phi[9], q[9], force[3], flow[3], lower[9];
    if (lsm3_coefficients(a1, a2, tl_h, dt, edge_opt, phi, q, force, flow)) { c->err = 1; return; }
    int factored = 0;
    double sigma_s = sigma_h;
    for (int d = 0; d < pd; d++) {
        double tl_k = tl_h;
        if (d == 2) {
            tl_k = tl_v;
            sigma_s = sigma_v;
            if (tl_v != tl_h) {
                if (lsm3_coefficients(a1, a2, tl_v, dt, edge_opt, phi, q, force, flow)) { c->err = 1; return; }
                factored = 0;
            }
        }
        double u_k = mean_flow[d];
        double Fp = d == 2 ? -GRAV * p->a0c : 0.;
        double ur0 = up0[d] - a2 * us0[d];
        double us_mean = (us0[d] * phi[0] + u_k * flow[0] + mean_acc[d] * tl_k * flow[0]);
        double ur_mean = (ur0 * phi[4] + us0[d] * phi[3] + u_k * flow[1] +
                          mean_acc[d] * tl_k * flow[1] + Fp * force[1]);
        double xp_mean = (xp0[d] + ur0 * force[1] + us0[d] * phi[6] + u_k * flow[2] +
                          mean_acc[d] * tl_k * flow[2] + Fp * force[2]);
        if (sigma_s > 0. && q[0] > 0.) {
            if (!factored) {
                if (edge_opt == 2) lsm3_cholesky_clipped(q, lower);
                else if (lsm3_cholesky(q, lower)) { c->err = 1; return; }
                factored = 1;
            }
            double xix, xiy, xiz;
            if (lower[4] > 0.) rng_pair(&c->rng, p->rng_method, &xix, &xiy);
            else { xix = rng_single(&c->rng, p->rng_method); xiy = 0.; }
            xiz = lower[8] > 0. ? rng_single(&c->rng, p->rng_method) : 0.;
            us_mean += sigma_s * lower[0] * xix;
            ur_mean += sigma_s * (lower[3] * xix + lower[4] * xiy);
            xp_mean += sigma_s * (lower[6] * xix + lower[7] * xiy + lower[8] * xiz);
        }
        FVS(c, d) = us_mean;
        VEL(c, d) = ur_mean + a2 * us_mean;
        POS(c, d) = xp_mean;
    }
}

/* update_state_lsm3.pyx:587-662 */
static int update_state_lsm3(ctx_t *c) {
    const cgo_params *p = c->p;
    int bnd_j = -1, i = c->i;
    for (int d = 0; d < c->pd; d++) { LPOS(c, d) = POS(c, d); LVEL(c, d) = VEL(c, d); }
    if (p->time_scheme == 1) euler_maruyama_lsm3(c);
    else if (p->time_scheme == 5) di_lsm3(c);
    else { c->err = 1; return -1; }
    c->s->last_tri[i] = c->s->tri[i];
    cgo_xy_localize(c->m, c->s->last_tri[i], LPOS(c, 0), LPOS(c, 1), POS(c, 0), POS(c, 1),
                    &c->s->tri[i], &bnd_j);
    if (c->pd == 3)
        c->s->lowerlayer[i] = z_localize(c->m, c->f, c->s->tri[i], POS(c, 0), POS(c, 1), POS(c, 2));
    return bnd_j;
}

/* init_lsm3_fluctuations.pyx:28-90 */
static void lsm3_fluctuations(ctx_t *c, double *f1, double *f2, double *f3) {
    const cgo_params *p = c->p;
    int diffmod = p->diffusion_model;
    double sigma_h, sigma_v, kt, ep;
    *f1 = *f2 = *f3 = 0.;
    if (diffmod == 2 || diffmod == 3) {
        double z = c->pd == 3 ? POS(c, 2) : 0.;
        if (turb_fields(c, c->s->tri[c->i], c->s->lowerlayer[c->i], POS(c, 0), POS(c, 1), z, &kt, &ep))
            c->err = 1;
        ep = fmax(ep, EPSILON);
        double tml = fmax(EPSILON_LSM3, (kt / ep) / (0.5 + (3. / 4.) * C0KOLM));
        sigma_h = sqrt(0.5 * C0KOLM * ep * tml);
    } else {
        sigma_h = sqrt(p->nux / p->tl_h);
    }
    if (sigma_h > 0.) {
        double xix, xiy;
        rng_pair(&c->rng, p->rng_method, &xix, &xiy);
        *f1 = sigma_h * xix;
        *f2 = sigma_h * xiy;
    }
    if (c->pd == 3) {
        sigma_v = diffmod == 3 ? sigma_h : sqrt(p->nuz / p->tl_v);
        if (sigma_v > 0.) *f3 = sigma_v * rng_single(&c->rng, p->rng_method);
    }
}

/* ======================================================================
 * Boundary conditions (cylag/boundary_conditions/compute_bc.pyx:35-395)
 * ====================================================================== */

/* utils.pyx:99-119 */
static void normal2u(double v0x, double v0y, double v1x, double v1y, double *nx, double *ny) {
    double norm = sqrt((v1x - v0x) * (v1x - v0x) + (v1y - v0y) * (v1y - v0y));
    *nx = (v0y - v1y) / norm;
    *ny = (v1x - v0x) / norm;
}

/* velocity reflection about the wall normal, compute_bc.pyx:190-240 */
static void reflect_velocity(ctx_t *c, double *vel, double ex0, double ey0,
                             double ex1, double ey1, double damp, int damp_vel,
                             double roughness) {
    double nx, ny;
    normal2u(ex0, ey0, ex1, ey1, &nx, &ny);
    if (c->p->bc_type == 2 && roughness > 0.) {
        double max_theta = 85.0 * DEG_TO_RAD;
        double theta = rng_single(&c->rng, c->p->rng_method) * roughness;
        theta = fmax(-max_theta, fmin(max_theta, theta));
        double ct = cos(theta), st = sin(theta);
        double nnx = nx * ct - ny * st;
        double nny = nx * st + ny * ct;
        nx = nnx; ny = nny;
    }
    double u0 = vel[0];
    vel[0] = u0 * nx + vel[1] * ny;
    vel[1] = -u0 * ny + vel[1] * nx;
    vel[0] = -1. * vel[0];
    u0 = vel[0];
    vel[0] = u0 * nx - vel[1] * ny;
    vel[1] = u0 * ny + vel[1] * nx;
    if (damp_vel) {
        vel[0] *= 1. - damp;
        vel[1] *= 1. - damp;
        if (c->pd == 3) vel[2] *= 1. - damp;
    }
}

/* control sections (control_shapes.pyx:74-101): the first segment
 * {x0, y0, x1, y1} of each; counts of the current cgo_step call */
static int g_ncsec = 0;
static double g_csec[4 * 64];
static int32_t g_csec_counts[64];

int cgo_set_sections(int n, const double *seg) {
    if (n < 0 || n > 64) return -1;
    g_ncsec = n;
    if (n) memcpy(g_csec, seg, (size_t)n * 4 * sizeof(double));
    memset(g_csec_counts, 0, sizeof g_csec_counts);
    return 0;
}

void cgo_take_section_counts(int32_t *out) {
    memcpy(out, g_csec_counts, (size_t)g_ncsec * sizeof(int32_t));
    memset(g_csec_counts, 0, sizeof g_csec_counts);
}

/* stranding output (compute_bc.pyx:109-121): {index, x, y, z} of each
 * stranded particle of the current cgo_step call, in any order (the caller
 * sorts by index, the reference's loop order) */
static int g_strand_on = 0;
static double *g_strand = NULL;
static int g_strand_n = 0, g_strand_cap = 0;

void cgo_set_stranding(int on) {
    g_strand_on = on;
    g_strand_n = 0;
}

int cgo_take_stranded(double *out, int cap) {
    int n = g_strand_n < cap ? g_strand_n : cap;
    if (out) memcpy(out, g_strand, (size_t)n * 4 * sizeof(double));
    g_strand_n = 0;
    return n;
}

static void record_strand(int i, double x, double y, double z) {
#pragma omp critical(cgo_strand)
    {
        if (g_strand_n == g_strand_cap) {
            int cap = g_strand_cap ? 2 * g_strand_cap : 256;
            double *b = (double *)realloc(g_strand, (size_t)cap * 4 * sizeof(double));
            if (b) {
                g_strand = b;
                g_strand_cap = cap;
            }
        }
        if (g_strand_n < g_strand_cap) {
            double *r = g_strand + 4 * (size_t)g_strand_n++;
            r[0] = i;
            r[1] = x;
            r[2] = y;
            r[3] = z;
        }
    }
}

static void compute_bc(ctx_t *c, int bnd_j, int32_t *bnd_stats) {
    const cgo_params *p = c->p;
    const cgo_mesh *m = c->m;
    const cgo_fields *f = c->f;
    cgo_particles *s = c->s;
    int i = c->i;
    double damp = fmin(p->damp_coef, 1.0 - EPSILON_REBOUND);
    double strand = p->strand_prob;
    double roughness = p->roughness_deg * DEG_TO_RAD;
    int strand_condition = 0;

    if (bnd_j != -1) {
        int lab = m->edge_labels[bnd_j];
        if (lab == BND_WALL_REF && strand > 0.)
            strand_condition = rng_uniform(&c->rng) < strand;
        if (strand_condition && g_strand_on)
            record_strand(i, POS(c, 0), POS(c, 1), c->pd == 3 ? POS(c, 2) : 0.0);
        if (lab == BND_WALL_REF && strand_condition == 0) {
            int bnd_jj = bnd_j, rebound_count = 0;
            while (s->tri[i] == PART_LOC_O && rebound_count < p->max_wall_rebounds) {
                int i0 = m->edges[2 * bnd_jj], i1 = m->edges[2 * bnd_jj + 1];
                double ex0 = m->x[i0], ey0 = m->y[i0], ex1 = m->x[i1], ey1 = m->y[i1];
                /* intersections.pyx:27-62: damped mirror about the edge */
                double coef = 1. - damp / 2.;
                double nx = ey0 - ey1, ny = ex1 - ex0;          /* utils.pyx normal2 */
                double norm2 = nx * nx + ny * ny;
                double ux = POS(c, 0) - ex0, uy = POS(c, 1) - ey0;
                double dist = ux * nx + uy * ny;
                double px = POS(c, 0) - 2. * ((dist * coef) / norm2) * nx;
                double py = POS(c, 1) - 2. * ((dist * coef) / norm2) * ny;
                POS(c, 0) = px;
                POS(c, 1) = py;
                cgo_xy_localize(m, s->last_tri[i], LPOS(c, 0), LPOS(c, 1), px, py,
                                &s->tri[i], &bnd_jj);
                if (s->tri[i] == PART_LOC_O && bnd_jj != -1 && m->edge_labels[bnd_jj] >= BND_OPEN_REF) {
                    if (p->bnd_statistics && bnd_stats) {
#ifdef _OPENMP
#pragma omp atomic
#endif
                        bnd_stats[m->edge_labels[bnd_jj] - 1] += 1;
                    }
                    delete_single(s, c->pd, i);
                    break;
                }
                if (p->model == 0 || p->model >= 2)
                    reflect_velocity(c, &VEL(c, 0), ex0, ey0, ex1, ey1, damp, 1, roughness);
                if (p->model == 3)
                    reflect_velocity(c, &FVS(c, 0), ex0, ey0, ex1, ey1, damp, 0, roughness);
                rebound_count += 1;
                if (s->tri[i] == PART_LOC_O && bnd_jj == -1) break;
            }
            if (c->pd == 3 && s->tri[i] != PART_LOC_O)
                s->lowerlayer[i] = z_localize(m, f, s->tri[i], POS(c, 0), POS(c, 1), POS(c, 2));
        }
        if (lab >= BND_OPEN_REF) {
            delete_single(s, c->pd, i);
            if (p->bnd_statistics && bnd_stats) {
#ifdef _OPENMP
#pragma omp atomic
#endif
                bnd_stats[lab - 1] += 1;
            }
        }
    }

    /* vertical boundary conditions, compute_bc.pyx:287-374 */
    if (c->pd == 3) {
        for (int side = 0; side < 2; side++) {
            int want = side == 0 ? PART_LOC_B : PART_LOC_A;
            if (!(s->lowerlayer[i] == want && s->tri[i] != PART_LOC_O)) continue;
            int k = s->tri[i];
            double zbp, zsp;
            if (f->dim == 2) {
                zbp = interp_field_2d(m, f, f->zb, k, 0, POS(c, 0), POS(c, 1));
                zsp = interp_field_2d(m, f, f->zs, k, 0, POS(c, 0), POS(c, 1));
            } else {
                zbp = interp_field_2d(m, f, f->zs, k, 0, POS(c, 0), POS(c, 1));
                zsp = interp_field_2d(m, f, f->zs, k, f->nlayers - 1, POS(c, 0), POS(c, 1));
            }
            double hp = fmax(0., zsp - zbp);
            if (side == 0) {
                double dz = fabs(zbp - POS(c, 2));
                POS(c, 2) = fmin(zbp + (1. - damp) * dz, zbp + 0.5 * hp);
            } else {
                double dz = fabs(POS(c, 2) - zsp);
                POS(c, 2) = fmax(zsp - (1. - damp) * dz, zsp - 0.5 * hp);
            }
            s->lowerlayer[i] = cgo_lower_layer_index(f->nlayers, zsp, zbp, POS(c, 2));
            double sg = side == 0 ? 1. : -1.;
            if (p->model >= 2) VEL(c, 2) = sg * fabs(VEL(c, 2)) * (1. - damp);
            if (p->model == 3) FVS(c, 2) = sg * fabs(FVS(c, 2)) * (1. - damp);
        }
    }

    /* compute_bc.pyx:378-395 */
    if (s->inactive[i] == 0) {
        if (s->tri[i] == PART_LOC_O) delete_single(s, c->pd, i);
        if (s->lowerlayer[i] == PART_LOC_B) delete_single(s, c->pd, i);
        if (s->lowerlayer[i] == PART_LOC_A) delete_single(s, c->pd, i);
    }
}

/* ======================================================================
 * Solver (cylag/core/solver.pyx)
 * ====================================================================== */

/* solver.pyx:238-379 */
static void init_particle(ctx_t *c) {
    const cgo_params *p = c->p;
    cgo_particles *s = c->s;
    int i = c->i;
    s->tri[i] = cgo_locate(c->m, POS(c, 0), POS(c, 1));
    if (s->tri[i] == -1) delete_single(s, c->pd, i);
    if (c->pd == 3 && s->inactive[i] == 0) {
        double zs, zb;
        int k = s->tri[i];
        zs = interp_field_2d(c->m, c->f, c->f->zs, k, c->f->nlayers - 1, POS(c, 0), POS(c, 1));
        if (c->f->dim == 2) zb = interp_field_2d(c->m, c->f, c->f->zb, k, 0, POS(c, 0), POS(c, 1));
        else zb = interp_field_2d(c->m, c->f, c->f->zs, k, 0, POS(c, 0), POS(c, 1));
        s->lowerlayer[i] = cgo_lower_layer_index(c->f->nlayers, zs, zb, POS(c, 2));
        if (POS(c, 2) < zb) POS(c, 2) = zb + EPSILON;
        if (POS(c, 2) > zs) POS(c, 2) = zs - EPSILON;
        /* solver.pyx:325-332 */
        if (p->compute_depth && s->depth) s->depth[i] = zs - POS(c, 2);
    }
    if (s->inactive[i] == 0 && p->particle_velocity_init == 1) {
        double ux, uy, uz;
        if (c->f->dim == 2) {
            interp_velocity_2d(c->m, c->f, s->tri[i], POS(c, 0), POS(c, 1), &ux, &uy);
            VEL(c, 0) = ux; VEL(c, 1) = uy; FVS(c, 0) = ux; FVS(c, 1) = uy;
        } else {
            if (interp_velocity_3d(c->m, c->f, s->tri[i], s->lowerlayer[i], POS(c, 0), POS(c, 1),
                                   POS(c, 2), &ux, &uy, &uz))
                c->err = 1;
            VEL(c, 0) = ux; VEL(c, 1) = uy; VEL(c, 2) = uz;
            FVS(c, 0) = ux; FVS(c, 1) = uy; FVS(c, 2) = uz;
        }
        if (p->model == 2 && p->diffusion_lsm2_option >= 2 && p->diffusion_model != 0) {
            double f1, f2, f3;
            if (lsm2_fluctuations(c, &f1, &f2, &f3)) c->err = 1;
            VEL(c, 0) += f1;
            VEL(c, 1) += f2;
            if (c->pd == 3) VEL(c, 2) += f3;
        }
        for (int d = 0; d < c->pd; d++) FVS(c, d) = VEL(c, d);
        if (p->model == 3) {
            double f1, f2, f3;
            lsm3_fluctuations(c, &f1, &f2, &f3);
            FVS(c, 0) += f1;
            FVS(c, 1) += f2;
            if (c->pd == 3) FVS(c, 2) += f3;
        }
    }
}

static int ctx_begin(ctx_t *c, const cgo_mesh *m, const cgo_fields *f, const cgo_params *p,
                     cgo_particles *s, int i) {
    c->m = m; c->f = f; c->p = p; c->s = s; c->i = i; c->pd = p->pdim; c->err = 0;
    c->rng.state = s->rng_state[i];
    c->rng.inc = s->rng_inc[i];
    return 0;
}

static int g_errors = 0;

int cgo_take_errors(void) {
    int e;
#pragma omp atomic capture
    { e = g_errors; g_errors = 0; }
    return e;
}

static void ctx_end(ctx_t *c) {
    c->s->rng_state[c->i] = c->rng.state;
    if (c->err) {
#pragma omp atomic
        g_errors += 1;
    }
}

int cgo_init_range(const cgo_mesh *m, const cgo_fields *f, const cgo_params *p,
                   cgo_particles *s, int i0, int i1) {
    int ndel = 0;
    zig_init();
    for (int i = i0; i < i1; i++) {
        if (s->inactive[i] != 0) continue;
        ctx_t c;
        ctx_begin(&c, m, f, p, s, i);
        init_particle(&c);
        ctx_end(&c);
        if (s->inactive[i]) ndel++;
    }
    return ndel;
}

/* solver.pyx:459-524 for one particle range */
int cgo_step_range(const cgo_mesh *m, const cgo_fields *f, const cgo_params *p,
                   cgo_particles *s, int i0, int i1, int32_t *bnd_stats) {
    int ndel = 0;
    zig_init();
    for (int i = i0; i < i1; i++) {
        if (s->inactive[i] != 0) continue;
        ctx_t c;
        ctx_begin(&c, m, f, p, s, i);
        if (s->tri[i] == -2) init_particle(&c);
        if (s->inactive[i] == 0) {
            int bnd_j = -1;
            if (p->model == 1) bnd_j = update_state_lsm1(&c);
            else if (p->model == 2) bnd_j = update_state_lsm2(&c);
            else if (p->model == 3) bnd_j = update_state_lsm3(&c);
            else c.err = 1;
            if (p->boundary_conditions == 1) {
                compute_bc(&c, bnd_j, bnd_stats);
            } else {
                if (s->tri[i] == PART_LOC_O) delete_single(s, c.pd, i);
                if (s->lowerlayer[i] == PART_LOC_B) delete_single(s, c.pd, i);
                if (s->lowerlayer[i] == PART_LOC_A) delete_single(s, c.pd, i);
            }
            /* solver.pyx:526-538: depth below the free surface */
            if (p->compute_depth && s->depth && s->inactive[i] == 0 && c.pd == 3) {
                int k = s->tri[i];
                double zs = interp_field_2d(m, f, f->zs, k, f->nlayers - 1, POS(&c, 0), POS(&c, 1));
                s->depth[i] = zs - POS(&c, 2);
            }
            /* control sections, solver.pyx:542-549 (zeroed arrays when the
             * step deleted the particle) */
            for (int cs = 0; cs < g_ncsec; cs++) {
                const double *g = g_csec + 4 * cs;
                if (intersec2d(s->last_pos[i * c.pd], s->last_pos[i * c.pd + 1],
                               s->pos[i * c.pd], s->pos[i * c.pd + 1], g[0], g[1], g[2], g[3])) {
#pragma omp atomic
                    g_csec_counts[cs] += 1;
                }
            }
        }
        ctx_end(&c);
        if (s->inactive[i]) ndel++;
    }
    return ndel;
}

int cgo_step(const cgo_mesh *m, const cgo_fields *f, const cgo_params *p,
             cgo_particles *s, int32_t *bnd_stats, int nthreads) {
    int ndel = 0;
    zig_init();
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
    int chunk = 4096;
    int nchunks = (s->n + chunk - 1) / chunk;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1) reduction(+:ndel)
    for (int b = 0; b < nchunks; b++) {
        int a = b * chunk, e = a + chunk < s->n ? a + chunk : s->n;
        ndel += cgo_step_range(m, f, p, s, a, e, bnd_stats);
    }
#else
    (void)nthreads;
    ndel = cgo_step_range(m, f, p, s, 0, s->n, bnd_stats);
#endif
    return ndel;
}
