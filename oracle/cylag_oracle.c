/*
 * cylag_oracle.c -- CPU restatement of CyLag's per-particle time step.
 *
 * TEST INFRASTRUCTURE ONLY (see cylag_oracle.h).  Plain C, scalar, FP64,
 * compiled with -ffp-contract=off so that every multiply and add rounds
 * separately, exactly as the reference's Cython-generated C does under gcc
 * -O2 on x86-64.  Expressions keep the reference's evaluation order.
 */
#include "cylag_oracle.h"

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

/* xylocalizer.pyx:338-435 */
static void path_walk(const cgo_mesh *m, int k, double p0x, double p0y,
                      double x, double y, int *new_k_out, int *bnd_out) {
    int new_k = -1, niter = 0, niter_max = 50, intersected_edge = -1;
    while (new_k == -1 && niter <= niter_max) {
        int intersects = 0;
        for (int i = 0; i < 3; i++) {
            int j = m->triedge[3 * k + i];
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
    int kk = k < 0 ? k + m->nt : k;
    path_walk(m, kk, p0x, p0y, x, y, &nk, bnd_j);
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

/* mean velocity at (k, ll, x, y, z), update_state_lsm1.pyx:144-163 */
static void lsm1_velocity(ctx_t *c, int k, int ll, double x, double y, double z,
                          double *ux, double *uy, double *uz) {
    if (c->f->dim == 2) {
        interp_velocity_2d(c->m, c->f, k, x, y, ux, uy);
        *uz = 0.;
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

/* solver.pyx:238-379 (LSM1 subset: no LSM2/LSM3 fluctuation draws) */
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
        for (int d = 0; d < c->pd; d++) FVS(c, d) = VEL(c, d);
    }
}

static int ctx_begin(ctx_t *c, const cgo_mesh *m, const cgo_fields *f, const cgo_params *p,
                     cgo_particles *s, int i) {
    c->m = m; c->f = f; c->p = p; c->s = s; c->i = i; c->pd = p->pdim; c->err = 0;
    c->rng.state = s->rng_state[i];
    c->rng.inc = s->rng_inc[i];
    return 0;
}

static void ctx_end(ctx_t *c) {
    c->s->rng_state[c->i] = c->rng.state;
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
            else c.err = 1;
            if (p->boundary_conditions == 1) {
                compute_bc(&c, bnd_j, bnd_stats);
            } else {
                if (s->tri[i] == PART_LOC_O) delete_single(s, c.pd, i);
                if (s->lowerlayer[i] == PART_LOC_B) delete_single(s, c.pd, i);
                if (s->lowerlayer[i] == PART_LOC_A) delete_single(s, c.pd, i);
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
