/*
 * vpm_oracle.c -- CPU oracle for the UJ hot path.  TEST INFRASTRUCTURE ONLY
 * (see vpm_oracle.h).  Restates FLOWVPM.jl v4.0.3 in C; each function cites the
 * reference file:line it follows.  Compile with -ffp-contract=off.
 */
#include "vpm_oracle.h"
#include "../include/vpm_gb300.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/FLOWVPM.jl:62-66 */
#define PI_ 3.14159265358979323846
static const double const1 = 0.063493635934240969;   /* 1/(2*pi)^1.5 */
static const double const2 = 0.79788456080286541;    /* sqrt(2/pi)   */
static const double const3 = 0.23873241463784300;    /* 3/(4*pi)     */
static const double const4 = 0.079577471545947673;   /* 1/(4*pi)     */
static const double sqr2   = 1.4142135623730951;     /* sqrt(2)      */

/* Rows of the 46-row particle column (0-based here), src/FLOWVPM_particlefield.jl:239-252 */
enum { RX = 0, RG = 3, RSIG = 6, RVOL = 7, RCIRC = 8, RU = 9, RW = 12, RJ = 15, RPSE = 24,
       RM = 27, RC = 36, RSFS = 39, RSTATIC = 42, RUPREV = 43 };

#define COL(P, ld, i) ((P) + (int64_t)(ld) * (int64_t)(i))

static int set_threads(int nthreads)
{
#ifdef _OPENMP
    return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

/* ------------------------------------------------------------------ erf
 * custom_erf64, src/FLOWVPM_gpu_erf.jl:160-191.  Rational approximations of
 * fdlibm's s_erf.c (Sun Microsystems, freely distributable); the coefficient
 * tables are the published ones.  The reference evaluates erfc's exponential
 * as exp(-x*x - 0.5625 + R/S) (no split of x*x), and so does this. */
static const double erx = 8.45062911510467529297e-01;
static const double pp[5] = { 1.28379167095512558561e-01, -3.25042107247001499370e-01,
    -2.84817495755985104766e-02, -5.77027029648944159157e-03, -2.37630166566501626084e-05 };
static const double qq[6] = { 0.0, 3.97917223959155352819e-01, 6.50222499887672944485e-02,
    5.08130628187576562776e-03, 1.32494738004321644526e-04, -3.96022827877536812320e-06 };
static const double pa[7] = { -2.36211856075265944077e-03, 4.14856118683748331666e-01,
    -3.72207876035701323847e-01, 3.18346619901161753674e-01, -1.10894694282396677476e-01,
    3.54783043256182359371e-02, -2.16637559486879084300e-03 };
static const double qa[7] = { 0.0, 1.06420880400844228286e-01, 5.40397917702171048937e-01,
    7.18286544141962662868e-02, 1.26171219808761642112e-01, 1.36370839120290507362e-02,
    1.19844998467991074170e-02 };
static const double ra[8] = { -9.86494403484714822705e-03, -6.93858572707181764372e-01,
    -1.05586262253232909814e+01, -6.23753324503260060396e+01, -1.62396669462573470355e+02,
    -1.84605092906711035994e+02, -8.12874355063065934246e+01, -9.81432934416914548592e+00 };
static const double sa[9] = { 0.0, 1.96512716674392571292e+01, 1.37657754143519042600e+02,
    4.34565877475229228821e+02, 6.45387271733267880336e+02, 4.29008140027567833386e+02,
    1.08635005541779435134e+02, 6.57024977031928170135e+00, -6.04244152148580987438e-02 };
static const double rb[7] = { -9.86494292470009928597e-03, -7.99283237680523006574e-01,
    -1.77579549177547519889e+01, -1.60636384855821916062e+02, -6.37566443368389627722e+02,
    -1.02509513161107724954e+03, -4.83519191608651397019e+02 };
static const double sb[8] = { 0.0, 3.03380607434824582924e+01, 3.25792512996573918826e+02,
    1.53672958608443695994e+03, 3.19985821950859553908e+03, 2.55305040643316442583e+03,
    4.74528541206955367215e+02, -2.24409524465858183362e+01 };

static double sgn(double x) { return x > 0 ? 1.0 : (x < 0 ? -1.0 : x); }

double oracle_erf_ref(double x)
{
    double xabs = fabs(x), s = sgn(x), val = s * 1.0;
    if (xabs < 0.84375) {
        double z = x * x;
        double r = pp[0] + z * (pp[1] + z * (pp[2] + z * (pp[3] + z * pp[4])));
        double q = 1.0 + z * (qq[1] + z * (qq[2] + z * (qq[3] + z * (qq[4] + z * qq[5]))));
        double y = r / q;
        val = s * (xabs + xabs * y);
    } else if (xabs < 1.25) {
        double t = xabs - 1.0;
        double P = pa[0] + t * (pa[1] + t * (pa[2] + t * (pa[3] + t * (pa[4] + t * (pa[5] + t * pa[6])))));
        double Q = 1.0 + t * (qa[1] + t * (qa[2] + t * (qa[3] + t * (qa[4] + t * (qa[5] + t * qa[6])))));
        val = s * (erx + P / Q);
    } else if (xabs < 2.857142857142857) {
        double t = 1.0 / (x * x);
        double R = ra[0] + t * (ra[1] + t * (ra[2] + t * (ra[3] + t * (ra[4] + t * (ra[5] + t * (ra[6] + t * ra[7]))))));
        double S = 1.0 + t * (sa[1] + t * (sa[2] + t * (sa[3] + t * (sa[4] + t * (sa[5] + t * (sa[6] + t * (sa[7] + t * sa[8])))))));
        double r = exp(-x * x - 0.5625 + R / S);
        val = s * (1.0 - r / xabs);
    } else if (xabs < 6.0) {
        double t = 1.0 / (x * x);
        double R = rb[0] + t * (rb[1] + t * (rb[2] + t * (rb[3] + t * (rb[4] + t * (rb[5] + t * rb[6])))));
        double S = 1.0 + t * (sb[1] + t * (sb[2] + t * (sb[3] + t * (sb[4] + t * (sb[5] + t * (sb[6] + t * sb[7]))))));
        double r = exp(-x * x - 0.5625 + R / S);
        val = s * (1.0 - r / xabs);
    }
    return val;
}

static double erf_sel(double x, int erf_mode) { return erf_mode ? erf(x) : oracle_erf_ref(x); }

/* -------------------------------------------------------------- kernels
 * src/FLOWVPM_kernel.jl:45-84 */
static void g_dgdr_mode(int kernel, double r, double* g, double* dg, int erf_mode)
{
    switch (kernel) {
    case VPM_KERNEL_SINGULAR:          /* :48 */
        *g = 1.0; *dg = 0.0; break;
    case VPM_KERNEL_GAUSSIAN: {        /* :62-66 */
        double aux = exp(-r * r * r);
        *g = 1 - aux; *dg = 3 * r * r * aux; break;
    }
    case VPM_KERNEL_GAUSSIANERF: {     /* :53-57 */
        double aux = const2 * r * exp(-r * r / 2);
        *g = erf_sel(r / sqr2, erf_mode) - aux; *dg = r * aux; break;
    }
    case VPM_KERNEL_WINCKELMANS: {     /* :76-84 */
        double aux0 = r * r + 1;
        double aux02 = aux0 * aux0;
        aux0 = aux02 * aux02 * aux0;
        aux0 = sqrt(aux0);
        *g = r * r * r * (r * r + 2.5) / aux0;
        *dg = 7.5 * r * r / (aux0 * (r * r + 1));
        break;
    }
    default: *g = NAN; *dg = NAN;
    }
}

void oracle_g_dgdr(int kernel, double r, double* g, double* dg) { g_dgdr_mode(kernel, r, g, dg, 0); }

double oracle_zeta(int kernel, double r)
{
    switch (kernel) {
    case VPM_KERNEL_SINGULAR: return r == 0 ? 1.0 : 0.0;           /* :45 */
    case VPM_KERNEL_GAUSSIAN: return const3 * exp(-r * r * r);      /* :60 */
    case VPM_KERNEL_GAUSSIANERF: return const1 * exp(-r * r / 2);   /* :51 */
    case VPM_KERNEL_WINCKELMANS: {                                   /* :69-74 */
        double temp = r * r + 1;
        double temp2 = temp * temp * temp;
        temp = temp2 * temp2 * temp;
        return const4 * 7.5 / sqrt(temp);
    }
    default: return NAN;
    }
}

/* Neumaier-compensated accumulator */
typedef struct { double s, c; } csum;
static inline void cadd(csum* a, double x)
{
    double t = a->s + x;
    if (fabs(a->s) >= fabs(x)) a->c += (a->s - t) + x;
    else a->c += (x - t) + a->s;
    a->s = t;
}

/* ------------------------------------------------------------- UJ pairs
 * The P2P overload fmm.direct!, src/FLOWVPM_fmm.jl:102-168, evaluated per
 * target with sources in index order (the order of the reference's loop for
 * any one target).  Results go to a zeroed buffer that is then added to the
 * output, as buffer_to_target_system! does (src/FLOWVPM_fmm.jl:170-176). */
void oracle_uj_pairs(int64_t t0, int64_t t1, const double* xt,
                     int64_t ns, const double* xs, const double* gs, const double* sgs,
                     double* U, double* J, int kernel, int erf_mode, int compensated,
                     int nthreads)
{
    int nth = set_threads(nthreads);
    (void)nth;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nth)
    for (int64_t t = t0; t < t1; t++) {
        const double tx = xt[3 * t], ty = xt[3 * t + 1], tz = xt[3 * t + 2];
        double acc[12] = {0};
        csum cacc[12];
        memset(cacc, 0, sizeof(cacc));
        for (int64_t s = 0; s < ns; s++) {
            const double gamma_x = gs[3 * s], gamma_y = gs[3 * s + 1], gamma_z = gs[3 * s + 2];
            const double sigma = sgs[s];
            const double dx = tx - xs[3 * s];
            const double dy = ty - xs[3 * s + 1];
            const double dz = tz - xs[3 * s + 2];
            const double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 == 0) continue;                                   /* :118 */
            const double r = sqrt(r2);
            double g_sgm, dg_sgmdr;
            g_dgdr_mode(kernel, r / sigma, &g_sgm, &dg_sgmdr, erf_mode); /* :122 */
            const double r3inv = 1.0 / (r2 * r);
            const double crss1 = -const4 * r3inv * (dy * gamma_z - dz * gamma_y);
            const double crss2 = -const4 * r3inv * (dz * gamma_x - dx * gamma_z);
            const double crss3 = -const4 * r3inv * (dx * gamma_y - dy * gamma_x);
            const double aux = dg_sgmdr / (sigma * r) - 3 * g_sgm / r2;    /* :145 */
            const double aux2 = -const4 * g_sgm * r3inv;                   /* :148 */
            double v[12];
            v[0] = g_sgm * crss1; v[1] = g_sgm * crss2; v[2] = g_sgm * crss3;
            v[3]  = aux * crss1 * dx;                    /* du1x1 */
            v[4]  = aux * crss2 * dx - aux2 * gamma_z;   /* du2x1 */
            v[5]  = aux * crss3 * dx + aux2 * gamma_y;   /* du3x1 */
            v[6]  = aux * crss1 * dy + aux2 * gamma_z;   /* du1x2 */
            v[7]  = aux * crss2 * dy;                    /* du2x2 */
            v[8]  = aux * crss3 * dy - aux2 * gamma_x;   /* du3x2 */
            v[9]  = aux * crss1 * dz - aux2 * gamma_y;   /* du1x3 */
            v[10] = aux * crss2 * dz + aux2 * gamma_x;   /* du2x3 */
            v[11] = aux * crss3 * dz;                    /* du3x3 */
            if (compensated) {
                for (int k = 0; k < 12; k++) cadd(&cacc[k], v[k]);
            } else {
                for (int k = 0; k < 12; k++) acc[k] += v[k];
            }
        }
        if (compensated)
            for (int k = 0; k < 12; k++) acc[k] = cacc[k].s + cacc[k].c;
        for (int k = 0; k < 3; k++) U[3 * t + k] += acc[k];
        for (int k = 0; k < 9; k++) J[9 * t + k] += acc[3 + k];
    }
}

/* -------------------------------------------------------------- adjoint
 * g, g' = dg/drho and g'' of each kernel (derivatives of src/FLOWVPM_kernel.jl:45-84). */
void oracle_g_d1_d2(int kernel, double rho, double* g, double* d1, double* d2)
{
    switch (kernel) {
    case VPM_KERNEL_SINGULAR: *g = 1; *d1 = 0; *d2 = 0; break;
    case VPM_KERNEL_GAUSSIAN: {
        const double e = exp(-rho * rho * rho);
        *g = 1 - e; *d1 = 3 * rho * rho * e; *d2 = (6 * rho - 9 * rho * rho * rho * rho) * e; break;
    }
    case VPM_KERNEL_GAUSSIANERF: {
        const double e = exp(-rho * rho / 2);
        *g = erf(rho / sqr2) - const2 * rho * e;
        *d1 = const2 * rho * rho * e;
        *d2 = const2 * (2 * rho - rho * rho * rho) * e;
        break;
    }
    case VPM_KERNEL_WINCKELMANS: {
        const double q = rho * rho + 1;
        *g = rho * rho * rho * (rho * rho + 2.5) / pow(q, 2.5);
        *d1 = 7.5 * rho * rho / pow(q, 3.5);
        *d2 = 7.5 * rho * (2 - 5 * rho * rho) / pow(q, 4.5);
        break;
    }
    default: *g = *d1 = *d2 = NAN;
    }
}

/* Derivatives of phi = Ubar.u + Jbar:j for one pair (u, j of src/FLOWVPM_fmm.jl:112-160)
 * with respect to dx = x_t - x_s (out[0..2]), Gamma_s (out[3..5]) and sigma_s (out[6]).
 * With q(r) = -g(rho)/(4 pi r^3), A = q, B = q'/r, c = dx x Gamma:
 *   u = A c,   j_ab = B c_a dx_b + A eps_abl Gamma_l,
 *   phi = A P + B Q,  P = Ubar.c + wbar.Gamma,  Q = c.(Jbar dx),
 * wbar_l = eps_abl Jbar_ab. */
static void adj_pair(const double* dx, const double* G, double sigma, const double* Ub, const double* Jb,
                     int kernel, double* out)
{
    const double r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
    for (int k = 0; k < 7; k++) out[k] = 0;
    if (r2 == 0) return;
    const double r = sqrt(r2), rho = r / sigma;
    double g, g1, g2;
    oracle_g_d1_d2(kernel, rho, &g, &g1, &g2);
    const double r3 = r2 * r, r4 = r2 * r2, r5 = r4 * r;
    const double A = -const4 * g / r3;
    const double B = -const4 * (g1 / (sigma * r4) - 3 * g / r5);
    const double qpp = -const4 * (g2 / (sigma * sigma * r3) - 6 * g1 / (sigma * r4) + 12 * g / r5);
    const double Bpr = (qpp - B) / r2;                                  /* B'(r)/r */
    const double dA_ds = const4 * g1 * rho / (sigma * r3);
    const double dB_ds = -const4 * (2 * g1 - rho * g2) / (sigma * sigma * r4);
    double c[3] = {dx[1] * G[2] - dx[2] * G[1], dx[2] * G[0] - dx[0] * G[2], dx[0] * G[1] - dx[1] * G[0]};
    /* Jbar[a + 3b] = dL/dJ_ab ; JD = Jbar dx ; JTc = Jbar^T c */
    double JD[3], JTc[3];
    for (int a = 0; a < 3; a++) {
        JD[a] = Jb[a] * dx[0] + Jb[a + 3] * dx[1] + Jb[a + 6] * dx[2];
        JTc[a] = Jb[3 * a] * c[0] + Jb[3 * a + 1] * c[1] + Jb[3 * a + 2] * c[2];
    }
    const double wb[3] = {Jb[1 + 3 * 2] - Jb[2 + 3 * 1], Jb[2 + 3 * 0] - Jb[0 + 3 * 2], Jb[0 + 3 * 1] - Jb[1 + 3 * 0]};
    const double P = Ub[0] * c[0] + Ub[1] * c[1] + Ub[2] * c[2] + wb[0] * G[0] + wb[1] * G[1] + wb[2] * G[2];
    const double Q = c[0] * JD[0] + c[1] * JD[1] + c[2] * JD[2];
    /* dphi/d(dx) */
    const double s = B * P + Bpr * Q;
    const double GxU[3] = {G[1] * Ub[2] - G[2] * Ub[1], G[2] * Ub[0] - G[0] * Ub[2], G[0] * Ub[1] - G[1] * Ub[0]};
    const double GxJD[3] = {G[1] * JD[2] - G[2] * JD[1], G[2] * JD[0] - G[0] * JD[2], G[0] * JD[1] - G[1] * JD[0]};
    for (int k = 0; k < 3; k++) out[k] = s * dx[k] + A * GxU[k] + B * (GxJD[k] + JTc[k]);
    /* dphi/dGamma = A (Ubar x dx + wbar) + B (JD x dx) */
    const double Uxd[3] = {Ub[1] * dx[2] - Ub[2] * dx[1], Ub[2] * dx[0] - Ub[0] * dx[2], Ub[0] * dx[1] - Ub[1] * dx[0]};
    const double JDxd[3] = {JD[1] * dx[2] - JD[2] * dx[1], JD[2] * dx[0] - JD[0] * dx[2], JD[0] * dx[1] - JD[1] * dx[0]};
    for (int k = 0; k < 3; k++) out[3 + k] = A * (Uxd[k] + wb[k]) + B * JDxd[k];
    out[6] = dA_ds * P + dB_ds * Q;
}

void oracle_uj_adjoint(int64_t n, const double* x, const double* gam, const double* sig,
                       const double* Ubar, const double* Jbar, double* xbar, double* gbar,
                       double* sbar, int kernel, int nthreads)
{
    int nth = set_threads(nthreads);
    (void)nth;
    const int sing = kernel == VPM_KERNEL_SINGULAR;
    /* target side: xbar_t += sum_s dphi/d(dx) */
#pragma omp parallel for schedule(dynamic, 16) num_threads(nth)
    for (int64_t t = 0; t < n; t++) {
        double acc[3] = {0, 0, 0}, o[7];
        for (int64_t s = 0; s < n; s++) {
            const double dx[3] = {x[3 * t] - x[3 * s], x[3 * t + 1] - x[3 * s + 1], x[3 * t + 2] - x[3 * s + 2]};
            adj_pair(dx, gam + 3 * s, sing ? 1.0 : sig[s], Ubar + 3 * t, Jbar + 9 * t, kernel, o);
            for (int k = 0; k < 3; k++) acc[k] += o[k];
        }
        for (int k = 0; k < 3; k++) xbar[3 * t + k] += acc[k];
    }
    /* source side: xbar_s -= sum_t dphi/d(dx), gbar_s, sbar_s */
#pragma omp parallel for schedule(dynamic, 16) num_threads(nth)
    for (int64_t s = 0; s < n; s++) {
        double acc[7] = {0, 0, 0, 0, 0, 0, 0}, o[7];
        for (int64_t t = 0; t < n; t++) {
            const double dx[3] = {x[3 * t] - x[3 * s], x[3 * t + 1] - x[3 * s + 1], x[3 * t + 2] - x[3 * s + 2]};
            adj_pair(dx, gam + 3 * s, sing ? 1.0 : sig[s], Ubar + 3 * t, Jbar + 9 * t, kernel, o);
            for (int k = 0; k < 7; k++) acc[k] += o[k];
        }
        for (int k = 0; k < 3; k++) { xbar[3 * s + k] -= acc[k]; gbar[3 * s + k] += acc[3 + k]; }
        if (!sing) sbar[s] += acc[6];
    }
}

/* ----------------------------------------------------------------- Estr
 * Estr_direct (src/FLOWVPM_subfilterscale_models.jl:16-41) inside the driver
 * loop of :61-74: non-static targets, non-static sources in index order. */
void oracle_estr_pairs(int64_t t0, int64_t t1, const double* xt, const double* Jt,
                       const uint8_t* static_t,
                       int64_t ns, const double* xs, const double* gs, const double* sgs,
                       const double* Js, const uint8_t* static_s,
                       double* SFS, int kernel, int transposed, int nthreads)
{
    int nth = set_threads(nthreads);
    (void)nth;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nth)
    for (int64_t t = t0; t < t1; t++) {
        if (static_t && static_t[t]) continue;
        const double tx = xt[3 * t], ty = xt[3 * t + 1], tz = xt[3 * t + 2];
        const double* JT = Jt + 9 * t;
        double sfs0 = SFS[3 * t], sfs1 = SFS[3 * t + 1], sfs2 = SFS[3 * t + 2];
        for (int64_t s = 0; s < ns; s++) {
            if (static_s && static_s[s]) continue;
            const double dx = xs[3 * s] - tx, dy = xs[3 * s + 1] - ty, dz = xs[3 * s + 2] - tz;
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            const double* JS = Js + 9 * s;
            const double* GS = gs + 3 * s;
            double S1, S2, S3;
            if (transposed) {
                S1 = (JT[0] - JS[0]) * GS[0] + (JT[1] - JS[1]) * GS[1] + (JT[2] - JS[2]) * GS[2];
                S2 = (JT[3] - JS[3]) * GS[0] + (JT[4] - JS[4]) * GS[1] + (JT[5] - JS[5]) * GS[2];
                S3 = (JT[6] - JS[6]) * GS[0] + (JT[7] - JS[7]) * GS[1] + (JT[8] - JS[8]) * GS[2];
            } else {
                S1 = (JT[0] - JS[0]) * GS[0] + (JT[3] - JS[3]) * GS[1] + (JT[6] - JS[6]) * GS[2];
                S2 = (JT[1] - JS[1]) * GS[0] + (JT[4] - JS[4]) * GS[1] + (JT[7] - JS[7]) * GS[2];
                S3 = (JT[2] - JS[2]) * GS[0] + (JT[5] - JS[5]) * GS[1] + (JT[8] - JS[8]) * GS[2];
            }
            const double sigma_inv = 1.0 / sgs[s];
            const double zeta_sgm = oracle_zeta(kernel, r * sigma_inv) * sigma_inv * sigma_inv * sigma_inv;
            sfs0 += zeta_sgm * S1;
            sfs1 += zeta_sgm * S2;
            sfs2 += zeta_sgm * S3;
        }
        SFS[3 * t] = sfs0; SFS[3 * t + 1] = sfs1; SFS[3 * t + 2] = sfs2;
    }
}

/* ---------------------------------------------------------- Estr adjoint
 * Reverse mode of the self-induced Estr of one particle set
 * (src/FLOWVPM_subfilterscale_models.jl:16-92): for
 *     phi = sum_t Sbar_t . SFS_t,  SFS_t = sum_{s != t} zeta(r/sigma_s)/sigma_s^3 S_ts,
 *     S_ts = (J_t - J_s)^T Gamma_s (transposed) or (J_t - J_s) Gamma_s (classic),
 * over non-static targets and non-static sources (the reference's iterator),
 * the gradients with respect to x, Gamma, sigma and J are added to xb, gb, sb,
 * Jb.  Each pair is differentiated directly from the definition: with
 * z = zeta/sigma^3, dz/dr = zeta'/sigma^4, dz/dsigma = -(rho zeta' + 3 zeta)/sigma^4,
 * w = Sbar_t . S_ts and M = J_t - J_s (M[a][b] = J[a + 3b]):
 *     d/dx_t = w dz/dr dx/r = -d/dx_s  (0 at r = 0: zeta'(0) = 0),
 *     d/dsigma_s = w dz/dsigma,
 *     d/dGamma_s = z M Sbar_t (transposed) or z M^T Sbar_t (classic),
 *     d/dJ_t[a + 3b] = z Gamma_s[a] Sbar_t[b] (transposed) or z Sbar_t[a] Gamma_s[b]
 *                      (classic) = -d/dJ_s[a + 3b].
 * The self pair (zero in the forward, and with zero gradient) is skipped.  The
 * target-side and the source-side sums run as two loops, each parallel over
 * its own output particle. */
static double zeta_d1(int kernel, double rho)
{
    switch (kernel) {
    case VPM_KERNEL_GAUSSIAN: return -3.0 * rho * rho * oracle_zeta(kernel, rho);
    case VPM_KERNEL_GAUSSIANERF: return -rho * oracle_zeta(kernel, rho);
    case VPM_KERNEL_WINCKELMANS: return -7.0 * rho * oracle_zeta(kernel, rho) / (rho * rho + 1.0);
    default: return 0.0;   /* singular: zeta is an indicator of r == 0 */
    }
}

/* per-pair terms of the Estr adjoint (see above); t != s, both non-static */
static void estr_adj_pair(const double* x, const double* gam, const double* sig, const double* J,
                          const double* Sbar, int64_t t, int64_t s, int kernel, int transposed,
                          double dxt[3], double* dsig, double dgam[3], double dJt[9])
{
    const double dx[3] = {x[3 * t] - x[3 * s], x[3 * t + 1] - x[3 * s + 1], x[3 * t + 2] - x[3 * s + 2]};
    const double r = sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
    const double sg = sig[s], rho = r / sg;
    const double zt = oracle_zeta(kernel, rho), z1 = zeta_d1(kernel, rho);
    const double z = zt / (sg * sg * sg);
    const double z_r = z1 / (sg * sg * sg * sg);
    const double z_s = -(rho * z1 + 3.0 * zt) / (sg * sg * sg * sg);
    const double* G = gam + 3 * s;
    const double* Sb = Sbar + 3 * t;
    double M[3][3];
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) M[a][b] = J[9 * t + a + 3 * b] - J[9 * s + a + 3 * b];
    double S[3];
    for (int k = 0; k < 3; k++) {
        S[k] = 0.0;
        for (int i = 0; i < 3; i++) S[k] += (transposed ? M[i][k] : M[k][i]) * G[i];
    }
    const double w = Sb[0] * S[0] + Sb[1] * S[1] + Sb[2] * S[2];
    for (int k = 0; k < 3; k++) dxt[k] = r > 0.0 ? w * z_r * dx[k] / r : 0.0;
    *dsig = w * z_s;
    for (int i = 0; i < 3; i++) {
        dgam[i] = 0.0;
        for (int k = 0; k < 3; k++) dgam[i] += z * (transposed ? M[i][k] : M[k][i]) * Sb[k];
    }
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) dJt[a + 3 * b] = transposed ? z * G[a] * Sb[b] : z * Sb[a] * G[b];
}

void oracle_estr_adjoint(int64_t n, const double* x, const double* gam, const double* sig, const double* J,
                         const uint8_t* st, const double* Sbar, double* xb, double* gb, double* sb, double* Jb,
                         int kernel, int transposed, int nthreads)
{
    int nth = set_threads(nthreads);
    (void)nth;
    /* target side: x_t and J_t */
#pragma omp parallel for schedule(dynamic, 16) num_threads(nth)
    for (int64_t t = 0; t < n; t++) {
        if (st && st[t]) continue;
        double ax[3] = {0, 0, 0}, aJ[9] = {0};
        for (int64_t s = 0; s < n; s++) {
            if (s == t || (st && st[s])) continue;
            double dxt[3], dsig, dgam[3], dJt[9];
            estr_adj_pair(x, gam, sig, J, Sbar, t, s, kernel, transposed, dxt, &dsig, dgam, dJt);
            for (int k = 0; k < 3; k++) ax[k] += dxt[k];
            for (int k = 0; k < 9; k++) aJ[k] += dJt[k];
        }
        for (int k = 0; k < 3; k++) xb[3 * t + k] += ax[k];
        for (int k = 0; k < 9; k++) Jb[9 * t + k] += aJ[k];
    }
    /* source side: x_s, Gamma_s, sigma_s and J_s */
#pragma omp parallel for schedule(dynamic, 16) num_threads(nth)
    for (int64_t s = 0; s < n; s++) {
        if (st && st[s]) continue;
        double ax[3] = {0, 0, 0}, ag[3] = {0, 0, 0}, as = 0.0, aJ[9] = {0};
        for (int64_t t = 0; t < n; t++) {
            if (t == s || (st && st[t])) continue;
            double dxt[3], dsig, dgam[3], dJt[9];
            estr_adj_pair(x, gam, sig, J, Sbar, t, s, kernel, transposed, dxt, &dsig, dgam, dJt);
            for (int k = 0; k < 3; k++) { ax[k] -= dxt[k]; ag[k] += dgam[k]; }
            as += dsig;
            for (int k = 0; k < 9; k++) aJ[k] -= dJt[k];
        }
        for (int k = 0; k < 3; k++) { xb[3 * s + k] += ax[k]; gb[3 * s + k] += ag[k]; }
        sb[s] += as;
        for (int k = 0; k < 9; k++) Jb[9 * s + k] += aJ[k];
    }
}

/* zeta_direct(sources, targets, zeta), src/FLOWVPM_viscous.jl:467-488: the
 * basis-function (vorticity) field W_t += sum_s zeta(r/sigma_s)/sigma_s^3 Gamma_s
 * over every source, the self pair (r = 0) included; statics take part. */
void oracle_zeta_pairs(int64_t t0, int64_t t1, const double* xt, int64_t ns, const double* xs,
                       const double* gs, const double* sgs, double* W, int kernel, int nthreads)
{
    int nth = set_threads(nthreads);
    (void)nth;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nth)
    for (int64_t t = t0; t < t1; t++) {
        double w0 = W[3 * t], w1 = W[3 * t + 1], w2 = W[3 * t + 2];
        for (int64_t s = 0; s < ns; s++) {
            const double dX1 = xt[3 * t] - xs[3 * s];
            const double dX2 = xt[3 * t + 1] - xs[3 * s + 1];
            const double dX3 = xt[3 * t + 2] - xs[3 * s + 2];
            const double r = sqrt(dX1 * dX1 + dX2 * dX2 + dX3 * dX3);
            const double zeta_sgm = 1.0 / (sgs[s] * sgs[s] * sgs[s]) * oracle_zeta(kernel, r / sgs[s]);
            w0 += gs[3 * s] * zeta_sgm;
            w1 += gs[3 * s + 1] * zeta_sgm;
            w2 += gs[3 * s + 2] * zeta_sgm;
        }
        W[3 * t] = w0; W[3 * t + 1] = w1; W[3 * t + 2] = w2;
    }
}

/* ------------------------------------------------------- UJ_direct (46 rows) */
static int is_static(const double* p) { return p[RSTATIC] != 0; }

/* _reset_particles / _reset_particles_sfs, src/FLOWVPM_particlefield.jl:464-507 */
static void reset_particles(double* P, int64_t ld, int64_t np)
{
    for (int64_t i = 0; i < np; i++) {
        double* p = COL(P, ld, i);
        if (is_static(p)) continue;
        for (int k = RU; k < RPSE + 3; k++) p[k] = 0;   /* U, vorticity, J, PSE */
    }
}
static void reset_particles_sfs(double* P, int64_t ld, int64_t np)
{
    for (int64_t i = 0; i < np; i++) {
        double* p = COL(P, ld, i);
        if (is_static(p)) continue;
        p[RSFS] = p[RSFS + 1] = p[RSFS + 2] = 0;
    }
}

int oracle_uj_direct(double* P, int64_t ld, int64_t np, int kernel, int flags,
                     int erf_mode, int nthreads)
{
    if (!P || ld != VPM_NFIELDS || np < 0 || kernel < 0 || kernel > 3) return -1;
    if (flags & VPM_RESET) reset_particles(P, ld, np);               /* UJ.jl:27-29 */
    if (flags & VPM_RESET_SFS) reset_particles_sfs(P, ld, np);       /* UJ.jl:30-32 */
    if (np == 0) return 0;
    double* x = malloc(sizeof(double) * 3 * np);
    double* gm = malloc(sizeof(double) * 3 * np);
    double* sg = malloc(sizeof(double) * np);
    double* U = calloc(3 * np, sizeof(double));
    double* J = calloc(9 * np, sizeof(double));
    uint8_t* st = malloc(np);
    for (int64_t i = 0; i < np; i++) {                   /* source_system_to_buffer!, fmm.jl:62-75 */
        const double* p = COL(P, ld, i);
        for (int k = 0; k < 3; k++) { x[3 * i + k] = p[RX + k]; gm[3 * i + k] = p[RG + k]; }
        sg[i] = p[RSIG];
        st[i] = (uint8_t)is_static(p);
    }
    oracle_uj_pairs(0, np, x, np, x, gm, sg, U, J, kernel, erf_mode, 0, nthreads); /* UJ.jl:35 */
    for (int64_t i = 0; i < np; i++) {                   /* buffer_to_target_system!, fmm.jl:170-176 */
        double* p = COL(P, ld, i);
        for (int k = 0; k < 3; k++) p[RU + k] += U[3 * i + k];
        for (int k = 0; k < 9; k++) p[RJ + k] += J[9 * i + k];
    }
    if (flags & VPM_SFS) {                               /* UJ.jl:36 */
        double* Jall = malloc(sizeof(double) * 9 * np);
        double* S = malloc(sizeof(double) * 3 * np);
        for (int64_t i = 0; i < np; i++) {
            const double* p = COL(P, ld, i);
            for (int k = 0; k < 9; k++) Jall[9 * i + k] = p[RJ + k];
            for (int k = 0; k < 3; k++) S[3 * i + k] = p[RSFS + k];
        }
        oracle_estr_pairs(0, np, x, Jall, st, np, x, gm, sg, Jall, st, S, kernel,
                          (flags & VPM_TRANSPOSED) != 0, nthreads);
        for (int64_t i = 0; i < np; i++) {
            double* p = COL(P, ld, i);
            for (int k = 0; k < 3; k++) p[RSFS + k] = S[3 * i + k];
        }
        free(Jall); free(S);
    }
    free(x); free(gm); free(sg); free(U); free(J); free(st);
    return 0;
}

/* ------------------------------------------------------------ consumers */

/* stretching S under the transposed or classic scheme */
static void stretch(const double* J, const double* G, int transposed, double* S)
{
    if (transposed) {
        S[0] = J[0] * G[0] + J[1] * G[1] + J[2] * G[2];
        S[1] = J[3] * G[0] + J[4] * G[1] + J[5] * G[2];
        S[2] = J[6] * G[0] + J[7] * G[1] + J[8] * G[2];
    } else {
        S[0] = J[0] * G[0] + J[3] * G[1] + J[6] * G[2];
        S[1] = J[1] * G[0] + J[4] * G[1] + J[7] * G[2];
        S[2] = J[2] * G[0] + J[5] * G[1] + J[8] * G[2];
    }
}

/* src/FLOWVPM_timeintegration.jl:463-532 */
void oracle_update_particle_states(double* P, int64_t ld, int64_t np, double a, double b,
                                   double dt, const double* Uinf, double f, double g,
                                   double zeta0, int transposed)
{
    for (int64_t i = 0; i < np; i++) {
        double* p = COL(P, ld, i);
        if (is_static(p)) continue;
        const double C = p[RC];
        double* M = p + RM;
        double* G = p + RG;
        const double* J = p + RJ;
        const double* U = p + RU;
        const double* SFS = p + RSFS;
        M[0] = a * M[0] + dt * (U[0] + Uinf[0]);
        M[1] = a * M[1] + dt * (U[1] + Uinf[1]);
        M[2] = a * M[2] + dt * (U[2] + Uinf[2]);
        p[RX] += b * M[0];
        p[RX + 1] += b * M[1];
        p[RX + 2] += b * M[2];
        double MM[3];
        stretch(J, G, transposed, MM);
        const double Gnorm2 = G[0] * G[0] + G[1] * G[1] + G[2] * G[2];
        const double sigma = p[RSIG];
        const double s3 = sigma * sigma * sigma;
        double MM4;
        if (Gnorm2 > 0) {
            MM4 = (f + g) / (1 + 3 * f) * (MM[0] * G[0] + MM[1] * G[1] + MM[2] * G[2]);
            MM4 -= f / (1 + 3 * f) * (C * SFS[0] * G[0] + C * SFS[1] * G[1] + C * SFS[2] * G[2]) * s3 / zeta0;
            MM4 /= Gnorm2;
        } else {
            MM4 = 0;
        }
        M[3] = a * M[3] + dt * (MM[0] - 3 * MM4 * G[0] - C * SFS[0] * s3 / zeta0);
        M[4] = a * M[4] + dt * (MM[1] - 3 * MM4 * G[1] - C * SFS[1] * s3 / zeta0);
        M[5] = a * M[5] + dt * (MM[2] - 3 * MM4 * G[2] - C * SFS[2] * s3 / zeta0);
        M[7] = a * M[7] - dt * (sigma * MM4);
        G[0] += b * M[3];
        G[1] += b * M[4];
        G[2] += b * M[5];
        p[RSIG] += b * M[7];
    }
}

/* src/FLOWVPM_relaxation.jl:62-81 (pedrizzetti), :112-142 (corrected) */
void oracle_relax(double* P, int64_t ld, int64_t np, double rlxf, int corrected)
{
    for (int64_t i = 0; i < np; i++) {
        double* p = COL(P, ld, i);
        if (is_static(p)) continue;
        const double* J = p + RJ;
        double* G = p + RG;
        const double w1 = J[5] - J[7], w2 = J[6] - J[2], w3 = J[1] - J[3];
        const double nrmw = sqrt(w1 * w1 + w2 * w2 + w3 * w3);
        if (nrmw == 0) continue;
        const double nrmGamma = sqrt(G[0] * G[0] + G[1] * G[1] + G[2] * G[2]);
        double b2 = 0;
        if (corrected)
            b2 = 1 - 2 * (1 - rlxf) * rlxf * (1 - (G[0] * w1 + G[1] * w2 + G[2] * w3) / (nrmGamma * nrmw));
        G[0] = (1 - rlxf) * G[0] + rlxf * nrmGamma * w1 / nrmw;
        G[1] = (1 - rlxf) * G[1] + rlxf * nrmGamma * w2 / nrmw;
        G[2] = (1 - rlxf) * G[2] + rlxf * nrmGamma * w3 / nrmw;
        if (corrected) {
            const double d = sqrt(b2);
            G[0] /= d; G[1] /= d; G[2] /= d;
        }
    }
}

/* dynamicprocedure_pseudo3level_beforeUJ, src/FLOWVPM_subfilterscale.jl:447-539 */
static void dyn_before(double* P, int64_t ld, int64_t np, oracle_step_params* prm, int uj_flags)
{
    for (int64_t i = 0; i < np; i++) {
        double* p = COL(P, ld, i);
        if (!is_static(p)) p[RSIG] *= prm->alpha;
    }
    oracle_uj_direct(P, ld, np, prm->kernel, uj_flags | VPM_SFS | VPM_RESET | VPM_RESET_SFS,
                     prm->erf_mode, prm->nthreads);
    for (int64_t i = 0; i < np; i++) {
        double* p = COL(P, ld, i);
        if (is_static(p)) continue;
        for (int k = 0; k < 9; k++) p[RM + k] = 0;
    }
    for (int64_t i = 0; i < np; i++) {
        double* p = COL(P, ld, i);
        if (is_static(p)) continue;
        stretch(p + RJ, p + RG, prm->transposed, p + RM);
        p[RM + 3] = p[RSFS]; p[RM + 4] = p[RSFS + 1]; p[RM + 5] = p[RSFS + 2];
    }
    for (int64_t i = 0; i < np; i++) {
        double* p = COL(P, ld, i);
        if (!is_static(p)) p[RSIG] /= prm->alpha;
    }
}

/* dynamicprocedure_pseudo3level_afterUJ, src/FLOWVPM_subfilterscale.jl:541-673 */
static int dyn_after(double* P, int64_t ld, int64_t np, oracle_step_params* prm, double zeta0)
{
    for (int64_t i = 0; i < np; i++) {
        double* p = COL(P, ld, i);
        if (is_static(p)) continue;
        double S[3];
        stretch(p + RJ, p + RG, prm->transposed, S);
        p[RM] -= S[0]; p[RM + 1] -= S[1]; p[RM + 2] -= S[2];
        p[RM + 3] -= p[RSFS]; p[RM + 4] -= p[RSFS + 1]; p[RM + 5] -= p[RSFS + 2];
    }
    int nan_found = 0;
    for (int64_t i = 0; i < np; i++) {
        double* p = COL(P, ld, i);
        if (is_static(p)) continue;
        const double* M = p + RM;
        double* Cp = p + RC;
        const double* G = p + RG;
        const double sigma = p[RSIG];
        double nume = M[0] * G[0] + M[1] * G[1] + M[2] * G[2];
        nume *= 3 * prm->alpha - 2;
        double deno = M[3] * G[0] + M[4] * G[1] + M[5] * G[2];
        deno /= zeta0 / (sigma * sigma * sigma);
        if (Cp[2] == 0) {
            Cp[2] = deno;
            if (Cp[2] == 0) Cp[2] = 2.220446049250313e-16;   /* eps() */
        }
        nume = prm->sfs_rlxf * nume + (1 - prm->sfs_rlxf) * Cp[1];
        deno = prm->sfs_rlxf * deno + (1 - prm->sfs_rlxf) * Cp[2];
        if (fabs(nume / deno) > prm->maxC) {
            if (fabs(deno) < fabs(Cp[2])) deno = sgn(deno) * fabs(Cp[2]);
            if (fabs(nume / deno) >= prm->maxC) nume = sgn(nume) * fabs(deno) * prm->maxC;
        } else if (fabs(nume / deno) < prm->minC) {
            nume = sgn(nume) * fabs(deno) * prm->minC;
        }
        Cp[1] = nume;
        Cp[2] = deno;
        Cp[0] = Cp[1] / Cp[2];
        if (isnan(Cp[0])) nan_found = 1;
        if (prm->force_positive) Cp[0] *= sgn(Cp[0]);
    }
    for (int64_t i = 0; i < np; i++) {
        double* p = COL(P, ld, i);
        if (is_static(p)) continue;
        for (int k = 0; k < 9; k++) p[RM + k] = 0;
    }
    return nan_found ? -3 : 0;
}

/* clipping_backscatter, src/FLOWVPM_subfilterscale.jl:282-296 */
static void clip_backscatter(double* P, int64_t ld, int64_t np)
{
    for (int64_t i = 0; i < np; i++) {
        double* p = COL(P, ld, i);
        if (is_static(p)) continue;
        const double C = p[RC];
        if (C * (p[RG] * p[RSFS] + p[RG + 1] * p[RSFS + 1] + p[RG + 2] * p[RSFS + 2]) < 0)
            p[RC] *= 0;
    }
}

/* rungekutta3 for ReformulatedVPM, src/FLOWVPM_timeintegration.jl:388-461, with
 * the SFS functors of src/FLOWVPM_subfilterscale.jl:113-268 and the RK3 branch
 * of the core-spreading scheme, src/FLOWVPM_viscous.jl:152-223. */
int oracle_rk3_step(double* P, int64_t ld, int64_t np, double dt, int relax,
                    oracle_step_params* prm)
{
    if (!P || ld != VPM_NFIELDS || np < 0) return -1;
    const int tflag = prm->transposed ? VPM_TRANSPOSED : 0;
    const int sfs_on = prm->sfs != 0;
    const double zeta0 = oracle_zeta(prm->kernel, 0.0);
    int rc = 0;
    for (int64_t i = 0; i < np; i++) {                              /* :401-414 */
        double* p = COL(P, ld, i);
        if (!is_static(p)) for (int k = 0; k < 9; k++) p[RM + k] = 0;
    }
    const double stages[3][2] = { {0.0, 1.0 / 3}, {-5.0 / 9, 15.0 / 16}, {-153.0 / 128, 8.0 / 15} };
    for (int st = 0; st < 3; st++) {
        const double a = stages[st][0], b = stages[st][1];
        const int first = (a == 1 || a == 0);
        if (prm->sfs == 2 && first) dyn_before(P, ld, np, prm, tflag);
        oracle_uj_direct(P, ld, np, prm->kernel,
                         VPM_RESET | tflag | (sfs_on ? (VPM_RESET_SFS | VPM_SFS) : 0),
                         prm->erf_mode, prm->nthreads);              /* :422 */
        if (prm->sfs == 2 && first) {
            rc = dyn_after(P, ld, np, prm, zeta0);
            if (rc) return rc;
            if (prm->clip_backscatter) clip_backscatter(P, ld, np);
        } else if (prm->sfs == 1 && first) {
            for (int64_t i = 0; i < np; i++) {
                double* p = COL(P, ld, i);
                if (!is_static(p)) p[RC] = prm->Cs;
            }
            if (prm->clip_backscatter) {
                for (int64_t i = 0; i < np; i++) {
                    double* p = COL(P, ld, i);
                    if (is_static(p)) continue;
                    if (p[RC] * (p[RG] * p[RSFS] + p[RG + 1] * p[RSFS + 1] + p[RG + 2] * p[RSFS + 2]) < 0)
                        p[RC] = 0;
                }
            }
        }
        oracle_update_particle_states(P, ld, np, a, b, dt, prm->Uinf, prm->f, prm->g, zeta0,
                                      prm->transposed);
        if (prm->viscous == 1) {                                     /* viscous.jl:175-220 */
            for (int64_t i = 0; i < np; i++) {
                double* p = COL(P, ld, i);
                if (is_static(p)) continue;
                p[RM + 6] = a * p[RM + 6] + dt * 2 * prm->nu;
                p[RSIG] = sqrt(p[RSIG] * p[RSIG] + b * p[RM + 6]);
            }
            if (fabs(b - 8.0 / 15) <= 1e-7) {
                prm->t_sgm += dt;
                const double beta_cur = sqrt(2 * prm->nu * prm->t_sgm / (prm->sgm0 * prm->sgm0) + 1);
                if (beta_cur >= prm->beta) return -2;
            }
        }
    }
    if (relax && prm->relaxation) {                                  /* :437-458 */
        reset_particles(P, ld, np);
        oracle_uj_direct(P, ld, np, prm->kernel, VPM_RESET | tflag, prm->erf_mode, prm->nthreads);
        oracle_relax(P, ld, np, prm->rlxf, prm->relaxation == 2);
    }
    return rc;
}
