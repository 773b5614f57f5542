/*
 * gi_oracle.h -- CPU oracle for the Giant-Impact force / kick-drift path.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only the tests, the smoke check in
 * __graft_entry__.py and the CPU-baseline leg of bench.py may load this
 * library; the product path (libgi.so) never links or calls it.
 *
 * Two restatements of the reference algorithm live here:
 *   - "ref-exact": FP32 pair arithmetic with the FP64 sub-expressions, the
 *     int truncation of dp.dv and the sequential j order of the reference
 *     kernels (Code/ImpactCode/impactAddTime.cu:245-394,
 *     Code/GenerateTargetImpactorCode/generateTargetImpactor.cu:486-664).
 *     Parallel over i with OpenMP; this is also the timed CPU baseline.
 *   - "fp64": the same pair law evaluated in double precision, the
 *     accuracy oracle every GPU result is measured against.
 */
#ifndef GI_ORACLE_H
#define GI_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Material/pair table.  Field order matches gi_pair_params in
 * include/gi_api.h so that one ctypes structure serves both. */
typedef struct gio_params {
    float GMassFeFe, GMassFeSi, GMassSiSi;
    float KFeFe, KSiSi, KFeSi;
    float KRFeFe, KRSiSi, KRFeSi, KRMix;
    float ShellBreakFe, ShellBreakSi, ShellBreakFeSi1, ShellBreakFeSi2;
    float MassFe, MassSi;
} gio_params;

/* One independent body set ("run"): bodies [offset, offset+n) interact only
 * with each other; the first nfe of them are Fe, the rest Si. */
typedef struct gio_run {
    int offset;
    int n;
    int nfe;
    int params;
    float dt, dt_over_mass_fe, dt_over_mass_si, damp;
} gio_run;

/* Separation test: 0 = reference (int)(dp.dv) > 0, 1 = dp.dv > 0. */
#define GIO_SEP_REF_INT 0
#define GIO_SEP_SIGN 1

/* Branch predicates of the fp64 oracle: 0 = evaluated exactly as the FP32
 * reference evaluates them (so that K/KR/band choices agree with the GPU),
 * 1 = evaluated in double. */
#define GIO_BRANCH_F32 0
#define GIO_BRANCH_F64 1

/* FMA contraction bits of the ref-exact restatement (nvcc contracts a*b+c
 * into fma by default).  bit0: r2, bit1: dp.dv, bit2: force accumulation,
 * bit3: move update. */
#define GIO_FMA_ALL 15

int gio_version(void);
int gio_max_threads(void);

/* Reference-exact force pass (float4 pos/vel/force arrays).  Writes only
 * force[i].xyz for i in the runs; .w untouched. */
void gio_forces_ref(const float *pos, const float *vel, float *force,
                    const gio_run *runs, int nruns, const gio_params *params,
                    int sep_test, int fma_mask, int nthreads);

/* Same, restricted to the i-bodies listed in idx (global indices); the
 * result for idx[k] goes to out[4k..4k+2]. */
void gio_forces_ref_subset(const float *pos, const float *vel, const int *idx,
                           int nidx, float *out, const gio_run *runs, int nruns,
                           const gio_params *params, int sep_test, int fma_mask,
                           int nthreads);

/* Reference-exact kick-drift (moveBodiesCollisionSingleGPU /
 * moveBodiesDampedSeperate): v += (F - damp v) dt/m, x += v dt. */
void gio_move_ref(float *pos, float *vel, const float *force,
                  const gio_run *runs, int nruns, int fma_mask, int nthreads);

/* FP64 oracle force for the listed i-bodies (idx NULL = every body of every
 * run, in order).  out is 3 doubles per listed body.  Also returns, per body,
 * sum_j |f_ij| in absf (may be NULL), the natural scale of its error. */
void gio_forces_fp64(const float *pos, const float *vel, const int *idx,
                     int nidx, double *out, double *absf,
                     const gio_run *runs, int nruns, const gio_params *params,
                     int sep_test, int branch_mode, int nthreads);

/* Pair potential energy per listed body, sum_{j != i} U(r_ij), in double.
 * U(r) = -Gm/r (r >= 1); -Gm + Gm(r-1) - K(r - r^3/3 - 2/3) (r < 1). */
void gio_potential_fp64(const float *pos, const int *idx, int nidx,
                        double *out, const gio_run *runs, int nruns,
                        const gio_params *params, int nthreads);

/* FP64 whole-run diagnostics over a run's bodies selected by label/scope:
 *   scope 0 = all, 1 = label 1 or 2, 2 = label 1, 3 = label 2
 * (label NULL = all bodies in every scope).  out[0..13]:
 *   mass, com xyz, vcom xyz, angular momentum about com (relative to vcom)
 *   xyz, kinetic energy, momentum xyz, count. */
void gio_diag_fp64(const float *pos, const float *vel,
                   const unsigned char *label, int scope,
                   const gio_run *run, const gio_params *params, double *out);

/* Count branch decisions that differ between FP32 (reference) and FP64
 * predicates over all pairs of the listed bodies: out[0] = band flips
 * (gravity / K / shell), out[1] = separation-test flips. */
void gio_count_flips(const float *pos, const float *vel, const int *idx,
                     int nidx, long long *out, const gio_run *runs, int nruns,
                     const gio_params *params, int sep_test, int nthreads);

/* FP64 trajectory of one run: the pair law in double, with double band and
 * separation decisions, on double positions and velocities (x, y, z per
 * body), integrated nsteps with the reference's kick-drift
 * (impactAddTime.cu:379-394) in double: v += F dt / m, then x += v dt.
 * Masses MassFe (the first nfe bodies) and MassSi.  At step 0 and every
 * `every` steps, log[7 k .. 7 k + 6] receives E = kinetic + pair potential
 * (the potential of gio_potential_fp64), L = sum m x cross v and
 * P = sum m v (x, y, z).  pos3 and vel3 are updated in place. */
void gio_integrate_fp64(double *pos3, double *vel3, int n, int nfe,
                        const gio_params *params, double dt, int nsteps, int every,
                        double *log, int sep_test, int nthreads);

/* Groups of touching bodies, restated literally from findEarthAndMoon
 * (Code/ImpactCode/impactBasicFunctions.h:109-155): group numbers are the
 * index of the body that started each group, the FP32 distance is
 * sqrtf((dx*dx + dy*dy) + dz*dz) < touch.  O(N^2); small N only.
 * group_id[i] receives body i's group number. */
void gio_groups_ref(const float *pos, int n, float touch, int *group_id);

/* The same groups by an independent method (cell lists of size 2*touch and
 * a sequential union-find that keeps the smallest index as the root). */
void gio_groups_uf(const float *pos, int n, float touch, int *group_id);

/* Earth / Moon choice and origin counts from group numbers
 * (impactBasicFunctions.h:157-216, :921-935): Earth = first group number
 * with the strictly largest size, Moon = first other with the strictly
 * largest size.  bounds = NFe1, NFe1 + NFe2, NFe1 + NFe2 + NSi1.
 * out[0..12] = earth, moon (-1 if none), n_earth, n_moon, number of
 * non-empty groups, earth counts [Fe1, Fe2, Si1, Si2], moon counts. */
void gio_earth_moon_ref(const int *group_id, int n, const int *bounds, int *out);

/* Smallest float t with sqrtf(t) >= s (the r2 threshold equivalent to the
 * reference's  s <= sqrt(r2)  comparison). */
float gio_r2_threshold(float s);

#ifdef __cplusplus
}
#endif
#endif
