/*
 * gi_oracle.c -- CPU oracle for the Giant-Impact force / kick-drift path.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, the smoke check in
 * __graft_entry__.py and the CPU-baseline leg of bench.py load this library,
 * and only as the checker or as the timed CPU baseline.
 *
 * Compile with -ffp-contract=off: every fused multiply-add of the
 * reference's nvcc build is written out below as an explicit fmaf(), so the
 * result does not depend on the host compiler's contraction policy (gcc on
 * aarch64 would otherwise contract a*b+c on its own).
 *
 * Reference followed (paths relative to the Giant-Impact project):
 *   pair law, collision kernel   Code/ImpactCode/impactAddTime.cu:245-377
 *   kick-drift                   Code/ImpactCode/impactAddTime.cu:379-394
 *   separate-body kernel         Code/GenerateTargetImpactorCode/generateTargetImpactor.cu:486-626
 *   damped kick-drift            Code/GenerateTargetImpactorCode/generateTargetImpactor.cu:628-664
 *   double diagnostics           Code/GenerateTargetImpactorCode/generateTargetImpactorBasicFunctions.h:29-237
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "gi_oracle.h"

typedef struct { float x, y, z, w; } f4;

int gio_version(void) { return 1; }

int gio_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static int pick_threads(int nthreads)
{
    if (nthreads > 0) return nthreads;
    return gio_max_threads();
}

/* Find the run holding global body index g (runs are few; linear scan). */
static const gio_run *run_of(const gio_run *runs, int nruns, int g)
{
    for (int r = 0; r < nruns; ++r)
        if (g >= runs[r].offset && g < runs[r].offset + runs[r].n) return &runs[r];
    return NULL;
}

float gio_r2_threshold(float s)
{
    if (!(s > 0.0f)) return 0.0f;
    float t = s * s;
    while (sqrtf(t) < s) t = nextafterf(t, INFINITY);
    while (t > 0.0f && sqrtf(nextafterf(t, -INFINITY)) >= s) t = nextafterf(t, -INFINITY);
    return t;
}

/* ------------------------------------------------------------------------ */
/* Reference-exact pair evaluation                                           */
/* ------------------------------------------------------------------------ */

/* r2 = dx*dx + dy*dy + dz*dz as the reference's nvcc build evaluates it:
 * each add is fused with the product that stands first in it, giving
 * fma(dz, dz, fma(dx, dx, dy*dy)); pinned bit for bit against the golden
 * vectors from the reference kernels (tests/golden). */
static inline float dot3_ref(float ax, float ay, float az, float bx, float by,
                             float bz, int fused)
{
    /* fused == 1: (a.x b.x + a.y b.y) + a.z b.z with both adds fused onto
     * the product that stands first in each add: fma(az, bz, fma(ax, bx, ay*by)).
     * fused == 2: the other pairing, fma(az, bz, fma(ay, by, ax*bx)). */
    if (fused == 1) return fmaf(az, bz, fmaf(ax, bx, ay * by));
    if (fused == 2) return fmaf(az, bz, fmaf(ay, by, ax * bx));
    float t = ax * bx;
    t = t + ay * by;
    return t + az * bz;
}

/* Separation test of the reference: int inout = dp.dv; KR when inout > 0.
 * The float->int conversion truncates toward zero (and saturates), so
 * inout > 0 exactly when dp.dv >= 1.0f; NaN converts to 0 (K). */
static inline int separating(float dpdv, int sep_test)
{
    if (sep_test == GIO_SEP_SIGN) return dpdv > 0.0f;
    return dpdv >= 1.0f;
}

/* force_mag of one pair, reference-exact (impactAddTime.cu:298-366).
 * test = (i is Fe) + (j is Fe).  The double literals of the reference make
 * 1.0/r2, 1.0 - K*(1.0 - r2) and G - K*(1.0 - r2) double expressions rounded
 * to float; GMass/r2 and 1.0f/r stay float. */
static inline float ref_force_mag(int test, float r2, float r, float dx,
                                  float dy, float dz, const f4 *vi,
                                  const f4 *vj, const gio_params *c,
                                  int sep_test, int fuse_dot)
{
    double r2d = (double)r2;
    if (test == 0) {
        if (1.0 <= (double)r) return (float)((double)c->GMassSiSi / r2d);
        if (c->ShellBreakSi <= r)
            return (float)((double)c->GMassSiSi - (double)c->KSiSi * (1.0 - r2d));
        float dpdv = dot3_ref(dx, dy, dz, vj->x - vi->x, vj->y - vi->y,
                              vj->z - vi->z, fuse_dot);
        double k = separating(dpdv, sep_test) ? (double)c->KRSiSi : (double)c->KSiSi;
        return (float)((double)c->GMassSiSi - k * (1.0 - r2d));
    } else if (test == 1) {
        if (1.0 <= (double)r) return c->GMassFeSi / r2;
        if (c->ShellBreakFeSi1 <= r)
            return (float)((double)c->GMassFeSi - (double)c->KFeSi * (1.0 - r2d));
        float dpdv = dot3_ref(dx, dy, dz, vj->x - vi->x, vj->y - vi->y,
                              vj->z - vi->z, fuse_dot);
        int sep = separating(dpdv, sep_test);
        double k;
        if (c->ShellBreakFeSi2 <= r) k = sep ? (double)c->KRMix : (double)c->KFeSi;
        else k = sep ? (double)c->KRFeSi : (double)c->KFeSi;
        return (float)((double)c->GMassFeSi - k * (1.0 - r2d));
    } else {
        if (1.0 <= (double)r) return c->GMassFeFe / r2;
        if (c->ShellBreakFe <= r)
            return (float)((double)c->GMassFeFe - (double)c->KFeFe * (1.0 - r2d));
        float dpdv = dot3_ref(dx, dy, dz, vj->x - vi->x, vj->y - vi->y,
                              vj->z - vi->z, fuse_dot);
        double k = separating(dpdv, sep_test) ? (double)c->KRFeFe : (double)c->KFeFe;
        return (float)((double)c->GMassFeFe - k * (1.0 - r2d));
    }
}

/* Force on body id from every body of its run, j in increasing order. */
static void ref_body(const f4 *pos, const f4 *vel, int id, const gio_run *run,
                     const gio_params *c, int sep_test, int fma_mask,
                     float out[3])
{
    /* bit 4 selects the alternative pairing of the fused dot products */
    const int alt = (fma_mask >> 4) & 1;
    const int fuse_r2 = (fma_mask & 1) ? 1 + alt : 0,
              fuse_dot = ((fma_mask >> 1) & 1) ? 1 + alt : 0,
              fuse_acc = (fma_mask >> 2) & 1;
    const f4 pi = pos[id];
    const f4 vi = vel[id];
    const int sw = run->offset + run->nfe;
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    for (int ids = run->offset; ids < run->offset + run->n; ++ids) {
        const f4 pj = pos[ids];
        float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
        float r2 = dot3_ref(dx, dy, dz, dx, dy, dz, fuse_r2);
        float r = sqrtf(r2);
        float invr = (id == ids) ? 0.0f : 1.0f / r;
        int test = (id < sw) + (ids < sw);
        float fm = ref_force_mag(test, r2, r, dx, dy, dz, &vi, &vel[ids], c,
                                 sep_test, fuse_dot);
        if (fuse_acc) {
            fx = fmaf(fm * dx, invr, fx);
            fy = fmaf(fm * dy, invr, fy);
            fz = fmaf(fm * dz, invr, fz);
        } else {
            fx = fx + fm * dx * invr;
            fy = fy + fm * dy * invr;
            fz = fz + fm * dz * invr;
        }
    }
    out[0] = fx; out[1] = fy; out[2] = fz;
}

void gio_forces_ref(const float *pos, const float *vel, float *force,
                    const gio_run *runs, int nruns, const gio_params *params,
                    int sep_test, int fma_mask, int nthreads)
{
    const f4 *P = (const f4 *)pos, *V = (const f4 *)vel;
    int total = 0;
    for (int r = 0; r < nruns; ++r) total += runs[r].n;
    int nt = pick_threads(nthreads);
    for (int r = 0; r < nruns; ++r) {
        const gio_run *run = &runs[r];
        const gio_params *c = &params[run->params];
        #pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
        for (int k = 0; k < run->n; ++k) {
            int id = run->offset + k;
            float o[3];
            ref_body(P, V, id, run, c, sep_test, fma_mask, o);
            force[4 * (size_t)id + 0] = o[0];
            force[4 * (size_t)id + 1] = o[1];
            force[4 * (size_t)id + 2] = o[2];
        }
    }
    (void)total;
}

void gio_forces_ref_subset(const float *pos, const float *vel, const int *idx,
                           int nidx, float *out, const gio_run *runs, int nruns,
                           const gio_params *params, int sep_test, int fma_mask,
                           int nthreads)
{
    const f4 *P = (const f4 *)pos, *V = (const f4 *)vel;
    int nt = pick_threads(nthreads);
    #pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
    for (int k = 0; k < nidx; ++k) {
        const gio_run *run = run_of(runs, nruns, idx[k]);
        float o[3] = {0.0f, 0.0f, 0.0f};
        if (run) ref_body(P, V, idx[k], run, &params[run->params], sep_test, fma_mask, o);
        out[4 * (size_t)k + 0] = o[0];
        out[4 * (size_t)k + 1] = o[1];
        out[4 * (size_t)k + 2] = o[2];
    }
}

void gio_move_ref(float *pos, float *vel, const float *force,
                  const gio_run *runs, int nruns, int fma_mask, int nthreads)
{
    const int fuse = (fma_mask >> 3) & 1;
    int nt = pick_threads(nthreads);
    for (int r = 0; r < nruns; ++r) {
        const gio_run *run = &runs[r];
        #pragma omp parallel for schedule(static) num_threads(nt)
        for (int k = 0; k < run->n; ++k) {
            size_t id = (size_t)(run->offset + k);
            float temp = (k < run->nfe) ? run->dt_over_mass_fe : run->dt_over_mass_si;
            float damp = run->damp;
            for (int a = 0; a < 3; ++a) {
                float v = vel[4 * id + a], f = force[4 * id + a];
                if (fuse) {
                    float t = fmaf(-damp, v, f);
                    v = fmaf(t, temp, v);
                    vel[4 * id + a] = v;
                    pos[4 * id + a] = fmaf(v, run->dt, pos[4 * id + a]);
                } else {
                    float t = f - damp * v;
                    v = v + t * temp;
                    vel[4 * id + a] = v;
                    pos[4 * id + a] = pos[4 * id + a] + v * run->dt;
                }
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* FP64 oracle                                                               */
/* ------------------------------------------------------------------------ */

/* Band of a pair: 0 gravity, 1 full-K band, 2 FeSi middle shell, 3 inner
 * shell.  Evaluated either the reference's FP32 way or in double. */
static inline int band_f32(int test, float r, const gio_params *c)
{
    if (1.0 <= (double)r) return 0;
    if (test == 0) return (c->ShellBreakSi <= r) ? 1 : 3;
    if (test == 2) return (c->ShellBreakFe <= r) ? 1 : 3;
    if (c->ShellBreakFeSi1 <= r) return 1;
    if (c->ShellBreakFeSi2 <= r) return 2;
    return 3;
}

static inline int band_f64(int test, double r, const gio_params *c)
{
    if (1.0 <= r) return 0;
    if (test == 0) return ((double)c->ShellBreakSi <= r) ? 1 : 3;
    if (test == 2) return ((double)c->ShellBreakFe <= r) ? 1 : 3;
    if ((double)c->ShellBreakFeSi1 <= r) return 1;
    if ((double)c->ShellBreakFeSi2 <= r) return 2;
    return 3;
}

static inline void class_consts(int test, const gio_params *c, double *g,
                                double *k, double *kr_mid, double *kr_in)
{
    if (test == 0) { *g = c->GMassSiSi; *k = c->KSiSi; *kr_mid = c->KRSiSi; *kr_in = c->KRSiSi; }
    else if (test == 1) { *g = c->GMassFeSi; *k = c->KFeSi; *kr_mid = c->KRMix; *kr_in = c->KRFeSi; }
    else { *g = c->GMassFeFe; *k = c->KFeFe; *kr_mid = c->KRFeFe; *kr_in = c->KRFeFe; }
}

static void fp64_body(const f4 *P, const f4 *V, int id, const gio_run *run,
                      const gio_params *c, int sep_test, int branch_mode,
                      double out[3], double *absf)
{
    const f4 pi = P[id], vi = V[id];
    const int sw = run->offset + run->nfe;
    double fx = 0.0, fy = 0.0, fz = 0.0, sa = 0.0;
    for (int ids = run->offset; ids < run->offset + run->n; ++ids) {
        if (ids == id) continue;
        const f4 pj = P[ids], vj = V[ids];
        double dx = (double)pj.x - pi.x, dy = (double)pj.y - pi.y, dz = (double)pj.z - pi.z;
        double r2 = dx * dx + dy * dy + dz * dz;
        double r = sqrt(r2);
        int test = (id < sw) + (ids < sw);
        double g, k, krm, kri;
        class_consts(test, c, &g, &k, &krm, &kri);
        int band, sep = 0;
        if (branch_mode == GIO_BRANCH_F32) {
            float fdx = pj.x - pi.x, fdy = pj.y - pi.y, fdz = pj.z - pi.z;
            float fr2 = dot3_ref(fdx, fdy, fdz, fdx, fdy, fdz, 1);
            band = band_f32(test, sqrtf(fr2), c);
            if (band >= 2) {
                float dpdv = dot3_ref(fdx, fdy, fdz, vj.x - vi.x, vj.y - vi.y,
                                      vj.z - vi.z, 1);
                sep = separating(dpdv, sep_test);
            }
        } else {
            band = band_f64(test, r, c);
            if (band >= 2) {
                double dpdv = dx * ((double)vj.x - vi.x) + dy * ((double)vj.y - vi.y) +
                              dz * ((double)vj.z - vi.z);
                sep = (sep_test == GIO_SEP_SIGN) ? (dpdv > 0.0) : (dpdv >= 1.0);
            }
        }
        double mag;
        if (band == 0) mag = g / r2;
        else if (band == 1) mag = g - k * (1.0 - r2);
        else if (band == 2) mag = g - (sep ? krm : k) * (1.0 - r2);
        else mag = g - (sep ? kri : k) * (1.0 - r2);
        double s = mag / r;
        fx += s * dx; fy += s * dy; fz += s * dz;
        sa += fabs(mag);
    }
    out[0] = fx; out[1] = fy; out[2] = fz;
    if (absf) *absf = sa;
}

void gio_forces_fp64(const float *pos, const float *vel, const int *idx,
                     int nidx, double *out, double *absf,
                     const gio_run *runs, int nruns, const gio_params *params,
                     int sep_test, int branch_mode, int nthreads)
{
    const f4 *P = (const f4 *)pos, *V = (const f4 *)vel;
    int nt = pick_threads(nthreads);
    if (!idx) {
        nidx = 0;
        for (int r = 0; r < nruns; ++r) nidx += runs[r].n;
    }
    #pragma omp parallel for schedule(dynamic, 8) num_threads(nt)
    for (int k = 0; k < nidx; ++k) {
        int id;
        if (idx) id = idx[k];
        else {
            int rem = k, r = 0;
            while (rem >= runs[r].n) { rem -= runs[r].n; ++r; }
            id = runs[r].offset + rem;
        }
        const gio_run *run = run_of(runs, nruns, id);
        double o[3] = {0.0, 0.0, 0.0}, a = 0.0;
        if (run) fp64_body(P, V, id, run, &params[run->params], sep_test, branch_mode, o, &a);
        out[3 * (size_t)k + 0] = o[0];
        out[3 * (size_t)k + 1] = o[1];
        out[3 * (size_t)k + 2] = o[2];
        if (absf) absf[k] = a;
    }
}

void gio_potential_fp64(const float *pos, const int *idx, int nidx,
                        double *out, const gio_run *runs, int nruns,
                        const gio_params *params, int nthreads)
{
    const f4 *P = (const f4 *)pos;
    int nt = pick_threads(nthreads);
    if (!idx) {
        nidx = 0;
        for (int r = 0; r < nruns; ++r) nidx += runs[r].n;
    }
    #pragma omp parallel for schedule(dynamic, 8) num_threads(nt)
    for (int k = 0; k < nidx; ++k) {
        int id;
        if (idx) id = idx[k];
        else {
            int rem = k, r = 0;
            while (rem >= runs[r].n) { rem -= runs[r].n; ++r; }
            id = runs[r].offset + rem;
        }
        const gio_run *run = run_of(runs, nruns, id);
        double u = 0.0;
        if (run) {
            const gio_params *c = &params[run->params];
            const int sw = run->offset + run->nfe;
            const f4 pi = P[id];
            for (int ids = run->offset; ids < run->offset + run->n; ++ids) {
                if (ids == id) continue;
                double dx = (double)P[ids].x - pi.x, dy = (double)P[ids].y - pi.y,
                       dz = (double)P[ids].z - pi.z;
                double r = sqrt(dx * dx + dy * dy + dz * dz);
                int test = (id < sw) + (ids < sw);
                double g, kk, krm, kri;
                class_consts(test, c, &g, &kk, &krm, &kri);
                if (r >= 1.0) u += -g / r;
                else u += -g + g * (r - 1.0) - kk * (r - r * r * r / 3.0 - 2.0 / 3.0);
            }
        }
        out[k] = u;
    }
}

static inline int in_scope(const unsigned char *label, size_t i, int scope)
{
    if (!label || scope == 0) return 1;
    unsigned char l = label[i];
    if (scope == 1) return l == 1 || l == 2;
    if (scope == 2) return l == 1;
    if (scope == 3) return l == 2;
    if (scope == 4) return l == 3;
    return 0;
}

void gio_diag_fp64(const float *pos, const float *vel,
                   const unsigned char *label, int scope,
                   const gio_run *run, const gio_params *params, double *out)
{
    const f4 *P = (const f4 *)pos, *V = (const f4 *)vel;
    const gio_params *c = &params[run->params];
    double m = 0.0, sx = 0.0, sy = 0.0, sz = 0.0, px = 0.0, py = 0.0, pz = 0.0,
           ke = 0.0, cnt = 0.0;
    for (int k = 0; k < run->n; ++k) {
        size_t i = (size_t)(run->offset + k);
        if (!in_scope(label, i, scope)) continue;
        double mi = (k < run->nfe) ? (double)c->MassFe : (double)c->MassSi;
        m += mi;
        sx += mi * P[i].x; sy += mi * P[i].y; sz += mi * P[i].z;
        px += mi * V[i].x; py += mi * V[i].y; pz += mi * V[i].z;
        ke += 0.5 * mi * ((double)V[i].x * V[i].x + (double)V[i].y * V[i].y +
                          (double)V[i].z * V[i].z);
        cnt += 1.0;
    }
    double cx = 0, cy = 0, cz = 0, vx = 0, vy = 0, vz = 0;
    if (m > 0.0) { cx = sx / m; cy = sy / m; cz = sz / m; vx = px / m; vy = py / m; vz = pz / m; }
    double lx = 0.0, ly = 0.0, lz = 0.0;
    for (int k = 0; k < run->n; ++k) {
        size_t i = (size_t)(run->offset + k);
        if (!in_scope(label, i, scope)) continue;
        double mi = (k < run->nfe) ? (double)c->MassFe : (double)c->MassSi;
        double rx = P[i].x - cx, ry = P[i].y - cy, rz = P[i].z - cz;
        double ux = V[i].x - vx, uy = V[i].y - vy, uz = V[i].z - vz;
        lx += (ry * uz - rz * uy) * mi;
        ly += -(rx * uz - rz * ux) * mi;
        lz += (rx * uy - ry * ux) * mi;
    }
    out[0] = m;
    out[1] = cx; out[2] = cy; out[3] = cz;
    out[4] = vx; out[5] = vy; out[6] = vz;
    out[7] = lx; out[8] = ly; out[9] = lz;
    out[10] = ke;
    out[11] = px; out[12] = py; out[13] = pz;
    out[14] = cnt;
}

void gio_count_flips(const float *pos, const float *vel, const int *idx,
                     int nidx, long long *out, const gio_run *runs, int nruns,
                     const gio_params *params, int sep_test, int nthreads)
{
    const f4 *P = (const f4 *)pos, *V = (const f4 *)vel;
    int nt = pick_threads(nthreads);
    long long band_flips = 0, sep_flips = 0;
    #pragma omp parallel for schedule(dynamic, 8) num_threads(nt) reduction(+ : band_flips, sep_flips)
    for (int k = 0; k < nidx; ++k) {
        int id = idx[k];
        const gio_run *run = run_of(runs, nruns, id);
        if (!run) continue;
        const gio_params *c = &params[run->params];
        const int sw = run->offset + run->nfe;
        const f4 pi = P[id], vi = V[id];
        for (int ids = run->offset; ids < run->offset + run->n; ++ids) {
            if (ids == id) continue;
            const f4 pj = P[ids], vj = V[ids];
            int test = (id < sw) + (ids < sw);
            float fdx = pj.x - pi.x, fdy = pj.y - pi.y, fdz = pj.z - pi.z;
            float fr2 = dot3_ref(fdx, fdy, fdz, fdx, fdy, fdz, 1);
            double dx = (double)pj.x - pi.x, dy = (double)pj.y - pi.y, dz = (double)pj.z - pi.z;
            double r = sqrt(dx * dx + dy * dy + dz * dz);
            int b32 = band_f32(test, sqrtf(fr2), c), b64 = band_f64(test, r, c);
            if (b32 != b64) ++band_flips;
            if (b32 >= 2 && b64 >= 2) {
                float d32 = dot3_ref(fdx, fdy, fdz, vj.x - vi.x, vj.y - vi.y, vj.z - vi.z, 1);
                double d64 = dx * ((double)vj.x - vi.x) + dy * ((double)vj.y - vi.y) +
                             dz * ((double)vj.z - vi.z);
                int s32 = separating(d32, sep_test);
                int s64 = (sep_test == GIO_SEP_SIGN) ? (d64 > 0.0) : (d64 >= 1.0);
                if (s32 != s64) ++sep_flips;
            }
        }
    }
    out[0] = band_flips;
    out[1] = sep_flips;
}

/* ------------------------------------------------------ FP64 trajectory -- */

static void fp64_log(const double *X, const double *V, const double *m, int n, int nfe,
                     const gio_params *c, double *out, int nt)
{
    double ke = 0.0, pe = 0.0, lx = 0.0, ly = 0.0, lz = 0.0, px = 0.0, py = 0.0, pz = 0.0;
    #pragma omp parallel for schedule(dynamic, 16) num_threads(nt) reduction(+ : pe)
    for (int i = 0; i < n; ++i) {
        double u = 0.0;
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            double dx = X[3 * j] - X[3 * i], dy = X[3 * j + 1] - X[3 * i + 1],
                   dz = X[3 * j + 2] - X[3 * i + 2];
            double r = sqrt(dx * dx + dy * dy + dz * dz);
            double g, kk, krm, kri;
            class_consts((i < nfe) + (j < nfe), c, &g, &kk, &krm, &kri);
            if (r >= 1.0) u += -g / r;
            else u += -g + g * (r - 1.0) - kk * (r - r * r * r / 3.0 - 2.0 / 3.0);
        }
        pe += u;
    }
    for (int i = 0; i < n; ++i) {
        const double *x = X + 3 * i, *v = V + 3 * i;
        ke += 0.5 * m[i] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        lx += m[i] * (x[1] * v[2] - x[2] * v[1]);
        ly += m[i] * (x[2] * v[0] - x[0] * v[2]);
        lz += m[i] * (x[0] * v[1] - x[1] * v[0]);
        px += m[i] * v[0]; py += m[i] * v[1]; pz += m[i] * v[2];
    }
    out[0] = ke + 0.5 * pe;
    out[1] = lx; out[2] = ly; out[3] = lz;
    out[4] = px; out[5] = py; out[6] = pz;
}

void gio_integrate_fp64(double *X, double *V, int n, int nfe, const gio_params *c,
                        double dt, int nsteps, int every, double *log, int sep_test,
                        int nthreads)
{
    int nt = pick_threads(nthreads);
    double *F = (double *)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    double *m = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; ++i) m[i] = (i < nfe) ? (double)c->MassFe : (double)c->MassSi;
    int rec = 0;
    if (every > 0) fp64_log(X, V, m, n, nfe, c, log + 7 * rec++, nt);
    for (int step = 1; step <= nsteps; ++step) {
        #pragma omp parallel for schedule(dynamic, 16) num_threads(nt)
        for (int i = 0; i < n; ++i) {
            double fx = 0.0, fy = 0.0, fz = 0.0;
            const double xi = X[3 * i], yi = X[3 * i + 1], zi = X[3 * i + 2];
            for (int j = 0; j < n; ++j) {
                if (j == i) continue;
                double dx = X[3 * j] - xi, dy = X[3 * j + 1] - yi, dz = X[3 * j + 2] - zi;
                double r2 = dx * dx + dy * dy + dz * dz;
                double r = sqrt(r2);
                int test = (i < nfe) + (j < nfe);
                double g, k, krm, kri;
                class_consts(test, c, &g, &k, &krm, &kri);
                int band = band_f64(test, r, c), sep = 0;
                if (band >= 2) {
                    double dpdv = dx * (V[3 * j] - V[3 * i]) + dy * (V[3 * j + 1] - V[3 * i + 1]) +
                                  dz * (V[3 * j + 2] - V[3 * i + 2]);
                    sep = (sep_test == GIO_SEP_SIGN) ? (dpdv > 0.0) : (dpdv >= 1.0);
                }
                double s;
                if (band == 0) {
                    s = g / (r2 * r);
                } else {
                    double kk = band == 1 ? k : (sep ? (band == 2 ? krm : kri) : k);
                    s = (g - kk * (1.0 - r2)) / r;
                }
                fx += s * dx; fy += s * dy; fz += s * dz;
            }
            F[3 * i] = fx; F[3 * i + 1] = fy; F[3 * i + 2] = fz;
        }
        for (int i = 0; i < n; ++i) {
            const double dtm = dt / m[i];
            for (int a = 0; a < 3; ++a) {
                V[3 * i + a] += F[3 * i + a] * dtm;
                X[3 * i + a] += V[3 * i + a] * dt;
            }
        }
        if (every > 0 && step % every == 0) fp64_log(X, V, m, n, nfe, c, log + 7 * rec++, nt);
    }
    free(F);
    free(m);
}

/* ------------------------------------------------------------- groups -- */

static inline int touching_ref(const f4 *P, int k, int j, float touch)
{
    /* host code of the reference: each product and sum rounded to float */
    float dx = P[k].x - P[j].x;
    float dy = P[k].y - P[j].y;
    float dz = P[k].z - P[j].z;
    float s = dx * dx;
    s = s + dy * dy;
    s = s + dz * dz;
    return sqrtf(s) < touch;
}

void gio_groups_ref(const float *pos, int n, float touch, int *group_id)
{
    const f4 *P = (const f4 *)pos;
    unsigned char *used = (unsigned char *)calloc((size_t)(n > 0 ? n : 1), 1);
    for (int i = 0; i < n; ++i) group_id[i] = -1;
    int group = 0;
    for (int i = 0; i < n; ++i) {
        if (group_id[i] == -1) {
            group_id[i] = group;
            int k = i;
            while (k < n) {
                if (group_id[k] == group && !used[k]) {
                    for (int j = i; j < n; ++j)
                        if (touching_ref(P, k, j, touch)) group_id[j] = group;
                    used[k] = 1;
                    k = i;
                } else {
                    ++k;
                }
            }
        }
        ++group; /* numbered by i even when i already had a group */
    }
    free(used);
}

static int uf_root(int *parent, int x)
{
    while (parent[x] != x) {
        parent[x] = parent[parent[x]];
        x = parent[x];
    }
    return x;
}

typedef struct { long long key; int idx; } cell_entry;

static int cmp_cell(const void *a, const void *b)
{
    const cell_entry *x = (const cell_entry *)a, *y = (const cell_entry *)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->idx - y->idx;
}

static long long cell_key(long long cx, long long cy, long long cz)
{
    /* 21 bits per axis after an offset; cells are clamped, so far bodies share edge cells */
    const long long off = 1 << 20;
    cx = cx < -off ? -off : (cx >= off ? off - 1 : cx);
    cy = cy < -off ? -off : (cy >= off ? off - 1 : cy);
    cz = cz < -off ? -off : (cz >= off ? off - 1 : cz);
    return ((cx + off) << 42) | ((cy + off) << 21) | (cz + off);
}

static long long cell_coord(float x, double inv)
{
    double f = floor((double)x * inv);
    if (!(f >= -1e9)) f = -1e9;
    if (f > 1e9) f = 1e9;
    return (long long)f;
}

void gio_groups_uf(const float *pos, int n, float touch, int *group_id)
{
    const f4 *P = (const f4 *)pos;
    if (n <= 0) return;
    int *parent = (int *)malloc((size_t)n * sizeof(int));
    cell_entry *cells = (cell_entry *)malloc((size_t)n * sizeof(cell_entry));
    const double inv = 1.0 / (2.0 * (double)touch);
    for (int i = 0; i < n; ++i) {
        parent[i] = i;
        cells[i].key = cell_key(cell_coord(P[i].x, inv), cell_coord(P[i].y, inv),
                                cell_coord(P[i].z, inv));
        cells[i].idx = i;
    }
    qsort(cells, (size_t)n, sizeof(cell_entry), cmp_cell);
    for (int i = 0; i < n; ++i) {
        const long long cx = cell_coord(P[i].x, inv), cy = cell_coord(P[i].y, inv),
                        cz = cell_coord(P[i].z, inv);
        for (int o = 0; o < 27; ++o) {
            const long long key = cell_key(cx + o % 3 - 1, cy + (o / 3) % 3 - 1, cz + o / 9 - 1);
            /* first entry with this key */
            int lo = 0, hi = n;
            while (lo < hi) {
                int mid = (lo + hi) / 2;
                if (cells[mid].key < key) lo = mid + 1; else hi = mid;
            }
            for (int s = lo; s < n && cells[s].key == key; ++s) {
                const int j = cells[s].idx;
                if (j <= i || !touching_ref(P, i, j, touch)) continue;
                int a = uf_root(parent, i), b = uf_root(parent, j);
                if (a == b) continue;
                if (a < b) parent[b] = a; else parent[a] = b;
            }
        }
    }
    for (int i = 0; i < n; ++i) group_id[i] = uf_root(parent, i);
    free(parent);
    free(cells);
}

void gio_earth_moon_ref(const int *group_id, int n, const int *bounds, int *out)
{
    int *size = (int *)calloc((size_t)(n > 0 ? n : 1), sizeof(int));
    for (int j = 0; j < n; ++j) size[group_id[j]]++;
    int earth = -1, n_earth = 0, moon = -1, n_moon = 0, groups = 0;
    for (int g = 0; g < n; ++g) {
        if (size[g] > 0) ++groups;
        if (size[g] > n_earth) { n_earth = size[g]; earth = g; }
    }
    for (int g = 0; g < n; ++g)
        if (size[g] > n_moon && g != earth) { n_moon = size[g]; moon = g; }
    for (int k = 0; k < 13; ++k) out[k] = 0;
    out[0] = earth; out[1] = moon; out[2] = n_earth; out[3] = n_moon; out[4] = groups;
    for (int j = 0; j < n; ++j) {
        int c = j < bounds[0] ? 0 : (j < bounds[1] ? 1 : (j < bounds[2] ? 2 : 3));
        if (group_id[j] == earth) out[5 + c]++;
        else if (group_id[j] == moon) out[9 + c]++;
    }
    free(size);
}
