/* C restatement of RAPTOR's per-pixel imaging path.
 *
 * TEST INFRASTRUCTURE ONLY: this is the oracle the CUDA engine is checked
 * against (and the CPU baseline it is timed beside where the reference
 * sources are not available).  The engine never links or calls it.
 *
 * The arithmetic follows the reference operation by operation where the
 * order changes rounding (metric, connection, the 64-term geodesic
 * contraction, the transfer update), so that on the same inputs the port and
 * the reference agree to rounding.  One deliberate difference: the camera's
 * MKS angle is found by a deterministic Newton iteration from theta/pi run
 * to convergence, instead of Newton with restarts from the global
 * subtract-with-carry RNG (newtonraphson.c:49-72, rcarry.c:29-53).  Both
 * find the same root of a monotone function; the reference stops at a
 * 1e-6 relative step, so the two differ by at most ~1e-12 in the camera
 * angle. */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Operation counting (tests/test_flop_count.py): compiled as C++ with
 * -DPORT_COUNT_FLOPS, `double` becomes a type that counts every arithmetic
 * operation and libm call, and the ray loop files the counts under ray
 * set-up, geodesic step, and transfer call (sampled or cut). */
#ifdef PORT_COUNT_FLOPS
#include "flopcount.hpp"
#define double cdouble
unsigned long long port_flop_counter = 0;
static unsigned long long flop_bucket[8];
#define FLOP_SNAP(v) unsigned long long v = port_flop_counter
#define FLOP_ADD(b, v) (flop_bucket[b] += port_flop_counter - (v))
extern "C" void port_flop_buckets(unsigned long long out[8], int reset)
{
    for (int i = 0; i < 8; i++) {
        out[i] = flop_bucket[i];
        if (reset)
            flop_bucket[i] = 0;
    }
}
#else
#define FLOP_SNAP(v)
#define FLOP_ADD(b, v)
#endif

#include "raptor_port.h"

/* constants.h:16-29, j_nu.c:15 (cgs) */
#define K_ECHARGE 4.8032068e-10
#define K_EMASS 9.1093826e-28
#define K_PMASS 1.67262171e-24
#define K_BOLTZ 1.3806505e-16
#define K_CLIGHT 2.99792458e10
#define K_PLANCK 6.6260693e-27
#define K_GGRAV 6.6742e-8
#define K_PI 3.14159265358979323846
#define K_E2C 7.695589048e-30
#define K_E2CH 1.161410e-03
/* parameters.h:163,170,182,184-185 */
#define K_RCAM 1.e4
#define K_MAX_ORDER 100
#define K_MAX_STEPS 1e5
#define K_CUTOFF_OUTER (K_RCAM * 1.01)
#define K_HORIZON_MARG 1e-1
#define K_SOURCE_DIST 2.6228263e22 /* parameters.h:144 */

typedef struct ray_ctx {
    const port_scene *s;
    double stopx1, stopx2;
    double cutoff_inner;
    double Ne_unit, B_unit, Rg;
    double cam_x2;
} ray_ctx;

/* ---- spacetime: MKS metric.c:94-137 ---- */
void port_metric_dd(const port_scene *s, const double X[4], double g[16])
{
    const double a = s->a, h = s->hslope, R0 = s->R0;
    double r = exp(X[1]) + R0;
    double th = K_PI * X[2] + 0.5 * (1. - h) * sin(2. * K_PI * X[2]);
    double sn = sin(th), s2 = sn * sn, cs = cos(th);
    double rho2 = r * r + a * a * cs * cs;
    double rfac = r - R0;
    double hfac = K_PI + (1. - h) * K_PI * cos(2. * K_PI * X[2]);
    memset(g, 0, 16 * sizeof(double));
    g[0] = (-1. + 2. * r / rho2);
    g[1] = (2. * r / rho2) * rfac;
    g[3] = (-2. * a * r * s2 / rho2);
    g[4] = g[1];
    g[5] = (1. + 2. * r / rho2) * rfac * rfac;
    g[7] = (-a * s2 * (1. + 2. * r / rho2)) * rfac;
    g[10] = rho2 * hfac * hfac;
    g[12] = g[3];
    g[13] = g[7];
    g[15] = s2 * (rho2 + a * a * s2 * (1. + 2. * r / rho2));
}

/* ---- spacetime: MKS inverse, metric.c:207-231 ---- */
void port_metric_uu(const port_scene *s, const double X[4], double g[16])
{
    const double a = s->a, h = s->hslope;
    double r = exp(X[1]) + s->R0;
    double th = K_PI * X[2] + 0.5 * (1. - h) * sin(2. * K_PI * X[2]);
    double sn = sin(th), s2 = sn * sn, cs = cos(th);
    double irho2 = 1. / (r * r + a * a * cs * cs);
    double hfac = K_PI + (1. - h) * K_PI * cos(2. * K_PI * X[2]);
    memset(g, 0, 16 * sizeof(double));
    g[0] = -1. - 2. * r * irho2;
    g[1] = 2. * irho2;
    g[4] = g[1];
    g[5] = irho2 * (r * (r - 2.) + a * a) / (r * r);
    g[7] = a * irho2 / r;
    g[10] = irho2 / (hfac * hfac);
    g[13] = g[7];
    g[15] = irho2 / s2;
}

/* ---- spacetime: analytic MKS Christoffel symbols, metric.c:538-638 ----
 * G[i*16 + j*4 + k] = Gamma^i_{jk} */
void port_connection(const port_scene *s, const double X[4], double G[64])
{
    const double a = s->a, h = s->hslope;
#define GM(i, j, k) G[(i) * 16 + (j) * 4 + (k)]
    double r = s->R0 + exp(X[1]);
    double r2 = r * r;
    double rp = exp(X[1]);
    double rp2 = rp * rp;
    double rpp = rp;
    double th = K_PI * X[2] + 0.5 * (1. - h) * sin(2. * K_PI * X[2]);
    double thp = K_PI * (1. + (1. - h) * cos(2. * K_PI * X[2]));
    double thp2 = thp * thp;
    double thpp = -2. * K_PI * K_PI * (1. - h) * sin(2. * K_PI * X[2]);
    double cs = cos(th), c2 = cs * cs, sn = sin(th);
    double s2 = sn * sn, s2th = sin(2. * th), cot = 1. / tan(th);
    double a2 = a * a;
    double Sg = r2 + a2 * c2, Sg2 = Sg * Sg;
    double Dl = r2 - 2. * r + a2;
    double A = Sg * Dl + 2. * r * (r2 + a2);
    double iS = 1. / Sg, iS2 = iS * iS, iS3 = iS * iS * iS;
    double B = (2. * r2 - Sg) * iS3;
    double C = r * iS - a2 * B * s2;

    GM(0, 0, 0) = 2. * r * B;
    GM(0, 0, 1) = (Sg + 2. * r) * B * rp;
    GM(0, 1, 0) = GM(0, 0, 1);
    GM(0, 0, 2) = -a2 * r * s2th * iS2 * thp;
    GM(0, 2, 0) = GM(0, 0, 2);
    GM(0, 0, 3) = -2. * a * r * B * s2;
    GM(0, 3, 0) = GM(0, 0, 3);
    GM(0, 1, 1) = 2. * (Sg + r) * B * rp2;
    GM(0, 1, 2) = GM(0, 0, 2) * rp;
    GM(0, 2, 1) = GM(0, 1, 2);
    GM(0, 1, 3) = -a * s2 * GM(0, 0, 1);
    GM(0, 3, 1) = GM(0, 1, 3);
    GM(0, 2, 2) = -2. * r2 * iS * thp2;
    GM(0, 2, 3) = -a * s2 * GM(0, 0, 2);
    GM(0, 3, 2) = GM(0, 2, 3);
    GM(0, 3, 3) = -2. * r * C * s2;

    GM(1, 0, 0) = Dl * B / rp;
    GM(1, 0, 1) = (Dl - Sg) * B;
    GM(1, 1, 0) = GM(1, 0, 1);
    GM(1, 2, 0) = 0;
    GM(1, 0, 2) = 0;
    GM(1, 0, 3) = -a * Dl * B * s2 / rp;
    GM(1, 3, 0) = GM(1, 0, 3);
    GM(1, 1, 1) = rpp / rp - (2. * Sg - Dl) * B * rp;
    GM(1, 1, 2) = -a2 * sn * cs * iS * thp;
    GM(1, 3, 2) = 0;
    GM(1, 2, 1) = GM(1, 1, 2);
    GM(1, 2, 3) = 0;
    GM(1, 1, 3) = a * (r * iS + (Sg - Dl) * B) * s2;
    GM(1, 3, 1) = GM(1, 1, 3);
    GM(1, 2, 2) = -r * Dl * iS / rp * thp2;
    GM(1, 3, 3) = -Dl * C * s2 / rp;

    GM(2, 0, 0) = iS * GM(0, 0, 2) / thp2;
    GM(2, 0, 1) = GM(2, 0, 0) * rp;
    GM(2, 1, 0) = GM(2, 0, 1);
    GM(2, 2, 0) = 0;
    GM(2, 0, 2) = 0;
    GM(2, 0, 3) = a * r * (r2 + a2) * s2th * iS3 / thp;
    GM(2, 3, 0) = GM(2, 0, 3);
    GM(2, 1, 1) = GM(2, 0, 0) * rp2;
    GM(2, 1, 2) = r * iS * rp;
    GM(2, 2, 1) = GM(2, 1, 2);
    GM(2, 1, 3) = a * sn * cs * (A + Sg * (Sg - Dl)) * iS3 * rp / thp;
    GM(2, 3, 1) = GM(2, 1, 3);
    GM(2, 3, 2) = 0;
    GM(2, 2, 3) = 0;
    GM(2, 2, 2) = thpp / thp + GM(1, 1, 2);
    GM(2, 3, 3) = -sn * cs * (Dl * Sg2 + 2. * r * (r2 + a2) * (r2 + a2)) * iS3 / thp;

    GM(3, 0, 0) = a * B;
    GM(3, 0, 1) = GM(3, 0, 0) * rp;
    GM(3, 1, 0) = GM(3, 0, 1);
    GM(3, 0, 2) = -2. * a * r * cot * iS2 * thp;
    GM(3, 2, 0) = GM(3, 0, 2);
    GM(3, 0, 3) = -a2 * B * s2;
    GM(3, 3, 0) = GM(3, 0, 3);
    GM(3, 1, 1) = GM(3, 0, 0) * rp2;
    GM(3, 1, 2) = -a * (Sg + 2. * r) * cot * iS2 * rp * thp;
    GM(3, 2, 1) = GM(3, 1, 2);
    GM(3, 1, 3) = C * rp;
    GM(3, 3, 1) = GM(3, 1, 3);
    GM(3, 2, 2) = -a * r * iS * thp2;
    GM(3, 2, 3) = (cot + a2 * r * s2th * iS2) * thp;
    GM(3, 3, 2) = GM(3, 2, 3);
    GM(3, 3, 3) = -a * C * s2;
#undef GM
}

/* ---- geodesic right-hand side, integrator.c:126-146 ---- */
static void geodesic_rhs(const port_scene *s, const double y[8], double f[8])
{
    double G[64];
    port_connection(s, y, G);
    double A[4] = {0., 0., 0., 0.};
    const double *U = y + 4;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            for (int k = 0; k < 4; k++)
                A[i] -= G[i * 16 + j * 4 + k] * U[j] * U[k];
    for (int i = 0; i < 4; i++) {
        f[i] = U[i];
        f[i + 4] = A[i];
    }
}

/* ---- RK4, integrator.c:13-41 (weights 1/2, 1/2, 1) ---- */
static void step_rk4(const port_scene *s, double y[8], double dt)
{
    static const double w[4] = {0.5, 0.5, 1., 0.};
    double dx[4][8], ys[8], f[8];
    memcpy(ys, y, sizeof ys);
    for (int q = 0; q < 4; q++) {
        geodesic_rhs(s, ys, f);
        for (int i = 0; i < 8; i++) {
            dx[q][i] = dt * f[i];
            ys[i] = y[i] + dx[q][i] * w[q];
        }
    }
    for (int i = 0; i < 8; i++)
        y[i] = y[i] + 1. / 6. * (dx[0][i] + dx[1][i] * 2. + dx[2][i] * 2. + dx[3][i]);
}

/* ---- RK2 midpoint, integrator.c:44-70 ---- */
static void step_rk2(const port_scene *s, double y[8], double dt)
{
    static const double w[2] = {0.5, 0.};
    double dx[2][8], ys[8], f[8];
    memcpy(ys, y, sizeof ys);
    for (int q = 0; q < 2; q++) {
        geodesic_rhs(s, ys, f);
        for (int i = 0; i < 8; i++) {
            dx[q][i] = dt * f[i];
            ys[i] = y[i] + dx[q][i] * w[q];
        }
    }
    for (int i = 0; i < 8; i++)
        y[i] = y[i] + dx[1][i];
}

/* ---- adaptive step, integrator.c:109-122 (negative: backward tracing) ---- */
static double step_size(double eps, const double X[4], const double U[4])
{
    const double tiny = 1.e-20 * 1.e-20;
    double d1 = eps / (fabs(U[1]) + tiny);
    double d2 = eps * fmin(X[2], 1. - X[2]) / (fabs(U[2]) + tiny);
    double d3 = eps / (fabs(U[3]) + tiny);
    double i1 = 1. / (fabs(d1) + tiny);
    double i2 = 1. / (fabs(d2) + tiny);
    double i3 = 1. / (fabs(d3) + tiny);
    return -fmax(1. / (i1 + i2 + i3), 1e-12);
}

/* ---- camera MKS angle: root of pi x + (1-h)/2 sin(2 pi x) = theta,
 *      the equation of newtonraphson.c:11-18, clamped as line 71 ---- */
static double camera_x2(double theta, double h)
{
    double x = theta / K_PI;
    for (int it = 0; it < 100; it++) {
        double f = K_PI * x + 0.5 * (1. - h) * sin(2. * K_PI * x) - theta;
        double fp = K_PI + K_PI * (1. - h) * cos(2. * K_PI * x);
        double nx = x - f / fp;
        if (nx == x || fabs(nx - x) <= 1e-16 * fabs(nx)) {
            x = nx;
            break;
        }
        x = nx;
    }
    return fmin(1., fmax(x, 0.));
}

double port_camera_x2(const port_scene *s)
{
    double mu0 = cos(s->inclination / 180. * K_PI);
    return camera_x2(acos(mu0), s->hslope);
}

/* ---- initial wave vector, metric.c:650-727 with BL_to_KS_u
 *      (GRmath.c:135-184) and the MKS theta map (newtonraphson.c:76-97) ---- */
static void init_photon(const ray_ctx *c, double alpha, double beta, double ph[8])
{
    const port_scene *s = c->s;
    const double a = s->a;
    double mu0 = cos(s->inclination / 180. * K_PI);
    double Xc[4] = {0., log(K_RCAM), acos(mu0), 90. / 180. * K_PI};
    double ll = -alpha * sqrt(1. - mu0 * mu0);
    double qq = beta * beta + mu0 * mu0 * (alpha * alpha - 1.);
    double L1 = ll, Q1 = qq;
    double sc2 = sin(Xc[2]) * sin(Xc[2]);
    double cc2 = cos(Xc[2]) * cos(Xc[2]);
    double kd[4], ku[4];
    kd[0] = -1.;
    kd[3] = L1;
    double sgn = (beta < 0.) ? -1. : (beta > 0.) ? 1. : 0.;
    kd[2] = sgn * sqrt(fabs(Q1 - L1 * L1 * (cc2 / sc2) + cc2));
    kd[1] = 0.;
    double r = K_RCAM, rf = r;
    double th = acos(mu0);
    double st = sin(th), ct = cos(th);
    double sig = r * r + a * a * ct * ct;
    double dl = r * r + a * a - 2. * r;
    double A = (r * r + a * a) * (r * r + a * a) - dl * a * a * st * st;
    double g11 = sig / dl * rf * rf;
    double gu00 = -A / (sig * dl);
    double gu03 = -2. * a * r / (sig * dl);
    double gu33 = (dl - a * a * st * st) / (sig * dl * st * st);
    double gu22 = 1. / sig;
    ku[0] = gu00 * kd[0] + gu03 * kd[3];
    ku[3] = gu33 * kd[3] + gu03 * kd[0];
    ku[2] = gu22 * kd[2];
    ku[1] = sqrt((-ku[0] * kd[0] - ku[2] * kd[2] - ku[3] * kd[3]) / g11);

    /* BL -> KS: only k^t and k^phi pick up k^r terms */
    double rc = exp(Xc[1]);
    double dc = rc * rc - 2. * rc + a * a;
    double t01 = 2. * rc / dc * rc;
    double t31 = a / dc * rc;
    double rplus = 1. + sqrt(1. - a * a), rmin = 1. - sqrt(1. - a * a);
    ph[0] = Xc[0] + (log(dc) + 1. / sqrt(1. - a * a) * log((rc - rplus) / (rc - rmin)));
    ph[1] = Xc[1];
    ph[2] = Xc[2];
    ph[3] = Xc[3] + (a / (2. * sqrt(1. - a * a)) * log((rc - rplus) / (rc - rmin)));
    ph[4] = ku[0] + t01 * ku[1];
    ph[5] = ku[1];
    ph[6] = ku[2];
    ph[7] = t31 * ku[1] + ku[3];

    /* KS theta -> MKS x2; the k^2 equation is linear, one division */
    ph[2] = c->cam_x2;
    ph[6] = ph[6] / (K_PI * (1. + (1. - s->hslope) * cos(2. * K_PI * ph[2])));
}

void port_init_photon(const port_scene *s, double alpha, double beta, double photon[8])
{
    ray_ctx c;
    memset(&c, 0, sizeof c);
    c.s = s;
    c.cam_x2 = port_camera_x2(s);
    init_photon(&c, alpha, beta, photon);
}

/* ---- thermal synchrotron emissivity, j_nu.c:130-153 (cos of pitch in) ---- */
double port_j_thsynch(double B, double costh, double thetae, double nu, double ne)
{
    double sth = sqrt(1 - costh * costh);
    double nuc = K_ECHARGE * B / (2. * K_PI * K_EMASS * K_CLIGHT);
    double nus = (2. / 9.) * nuc * thetae * thetae * sth;
    double X = nu / nus;
    double f = pow(pow(X, 0.5) + pow(2., 11. / 12.) * pow(X, 1. / 6.), 2.);
    if (nu == 1 || fabs(sth) < 1.e-10)
        return 0;
    if (!(thetae > 1e-4))
        return 0;
    double K2 = 2 * thetae * thetae;
    double j = ne * sqrt(2.) * K_PI * nus / (3. * K2) * f * exp(-pow(X, 1. / 3.));
    return j * K_E2C;
}

/* ---- Gauss hypergeometric function 2F1(a, b; c; x), in place of GSL's
 * gsl_sf_hyperg_2F1 at the kappa absorptivity's call sites (j_nu.c:85-96;
 * GSL is unpinned and absent here): the power series
 * sum_n (a)_n (b)_n / ((c)_n n!) x^n for 0 <= x <= 1/2, Pfaff's
 * transformation 2F1(a, b; c; x) = (1 - x)^-a 2F1(a, c - b; c; x / (x - 1))
 * for -1 <= x < 0 (which maps x into [0, 1/2]); the reference calls it only
 * on [-1, 1/2).  Checked against scipy's hyp2f1 by tests/test_oracle.py. ---- */
#ifndef PORT_COUNT_FLOPS /* the operation count covers the thermal path only */
double port_hyp2f1(double a, double b, double c, double x)
{
    if (x < 0)
        return pow(1 - x, -a) * port_hyp2f1(a, c - b, c, x / (x - 1));
    double term = 1.0, sum = 1.0;
    for (int n = 0; n < 400; n++) {
        term *= (a + n) * (b + n) / ((c + n) * (n + 1)) * x;
        sum += term;
        if (fabs(term) <= 1e-17 * fabs(sum))
            break;
    }
    return sum;
}

/* ---- kappa-distribution emissivity, j_nu.c:28-54 (kappa = 3.5; cos of pitch in) ---- */
double port_j_kappa(double nu, double ne, double thetae, double B, double costh)
{
    double kappa = 3.5;
    double w = thetae;
    double nuc = K_ECHARGE * B / (2. * K_PI * K_EMASS * K_CLIGHT);
    double sth = sqrt(1 - costh * costh);
    double factor = (ne * pow(K_ECHARGE, 2.) * nuc * sth) / K_CLIGHT;
    double nus = nuc * sth * pow(w * kappa, 2);
    if (nu == 1.0 || fabs(costh) == 1)
        return 0;
    double X = nu / nus;
    double J_low = pow(X, 1. / 3.) * 4 * K_PI * tgamma(kappa - 4. / 3.) / (pow(3, 7. / 3.) * tgamma(kappa - 2.));
    double J_high = pow(X, -(kappa - 2) / 2.) * pow(3, (kappa - 1) / 2.) * (kappa - 2.) * (kappa - 1.) / 4. *
                    tgamma(kappa / 4. - 1. / 3.) * tgamma(kappa / 4. + 4. / 3.);
    double x = 3 * pow(kappa, -3. / 2.);
    double J_s = pow((pow(J_low, -x) + pow(J_high, -x)), -1. / x);
    return J_s * factor;
}

/* ---- kappa-distribution absorptivity, j_nu.c:56-106 ---- */
double port_a_kappa(double nu, double ne, double thetae, double B, double costh)
{
    double kappa = 3.5;
    double w = thetae;
    double nuc = K_ECHARGE * B / (2. * K_PI * K_EMASS * K_CLIGHT);
    double sth = sqrt(1 - costh * costh);
    double factor = ne * K_ECHARGE / (B * sth);
    if (nu == 1.0 || fabs(costh) == 1.)
        return 0;
    double nus = nuc * sth * pow(w * kappa, 2);
    double X = nu / nus;
    double a = kappa - 1. / 3., b = kappa + 1., c = kappa + 2. / 3., z = -kappa * w;
    double hyp2F1;
    if (fabs(z) == 1.)
        return 0;
    if (fabs(z) > 1.)
        hyp2F1 = pow(1. - z, -a) * tgamma(c) * tgamma(b - a) / (tgamma(b) * tgamma(c - a)) *
                     port_hyp2f1(a, c - b, a - b + 1., 1. / (1. - z)) +
                 pow(1. - z, -b) * tgamma(c) * tgamma(a - b) / (tgamma(a) * tgamma(c - b)) *
                     port_hyp2f1(b, c - a, b - a + 1., 1. / (1. - z));
    else
        hyp2F1 = port_hyp2f1(a, b, c, z);
    double A_low = pow(X, -5. / 3.) * pow(3, 1. / 6.) * (10. / 41.) * pow(2 * K_PI, 2) / pow(w * kappa, 16. / 3. - kappa) *
                   (kappa - 2.) * (kappa - 1.) * kappa / (3. * kappa - 1.) * tgamma(5. / 3.) * hyp2F1;
    double A_high = pow(X, -(3. + kappa) / 2.) * (pow(K_PI, 5. / 2.) / 3.) *
                    ((kappa - 2.) * (kappa - 1.) * kappa / pow(w * kappa, 5.)) *
                    (2 * tgamma(2. + kappa / 2.) / (2. + kappa) - 1.) * (pow(3. / kappa, 19. / 4.) + 3. / 5.);
    double x = pow(-7. / 4. + 8. * kappa / 5., -43. / 50.);
    double A_s = pow((pow(A_low, -x) + pow(A_high, -x)), -1. / x);
    return factor * A_s;
}
#else
double port_j_kappa(double nu, double ne, double thetae, double B, double costh) { return 0.0 * (nu + ne + thetae + B + costh); }
double port_a_kappa(double nu, double ne, double thetae, double B, double costh) { return 0.0 * (nu + ne + thetae + B + costh); }
#endif

/* ---- Kirchhoff absorptivity with the Planck function, j_nu.c:188-200 ---- */
double port_a_th(double j, double nu, double thetae)
{
    double T = thetae * K_EMASS * K_CLIGHT * K_CLIGHT / K_BOLTZ;
    double Bnu = 2. * nu * nu * nu / (K_CLIGHT * K_CLIGHT) * 1. /
                 (exp(K_PLANCK * nu / (K_BOLTZ * T)) - 1.);
    return j * K_E2CH / Bnu / K_E2C;
}

static void lower(const double g[16], const double v[4], double out[4])
{
    for (int i = 0; i < 4; i++) {
        double acc = 0.;
        for (int j = 0; j < 4; j++)
            acc += g[i * 4 + j] * v[j];
        out[i] = acc;
    }
}

/* ---- plasma sampling, raptor_harm_model.c:190-320 with Xtoij and
 *      interp_scalar_2D (grmhd.c:35-71).  Returns 0 in the sigma > 1 cut. */
typedef struct fluid_state {
    double ne, thetae, B, beta;
    double bcon[4], ucon[4];
} fluid_state;

static int fluid_params(const ray_ctx *c, const double X[4], const double gcov[16],
                        const double gcon[16], fluid_state *fs)
{
    const port_scene *s = c->s;
    const double tiny = 1.e-20;
    int i = (int)((X[1] - s->startx1) / s->dx1 - 0.5);
    int j = (int)((X[2] - s->startx2) / s->dx2 - 0.5);
    double d1, d2;
    if (i < 0) {
        i = 0;
        d1 = 0.;
    } else if (i > s->n1 - 2) {
        i = s->n1 - 2;
        d1 = 1.;
    } else {
        d1 = (X[1] - ((i + 0.5) * s->dx1 + s->startx1)) / s->dx1;
    }
    if (j < 0) {
        j = 0;
        d2 = 0.;
    } else if (j > s->n2 - 2) {
        j = s->n2 - 2;
        d2 = 1.;
    } else {
        d2 = (X[2] - ((j + 0.5) * s->dx2 + s->startx2)) / s->dx2;
    }
    double cf[4] = {(1. - d1) * (1. - d2), (1. - d1) * d2, d1 * (1. - d2), d1 * d2};
    const size_t plane = (size_t)s->n1 * s->n2;
    const size_t at = (size_t)i * s->n2 + j;
    double v[8];
    for (int q = 0; q < 8; q++) {
        const double *P = s->prims + q * plane;
        v[q] = P[at] * cf[0] + P[at + 1] * cf[1] + P[at + s->n2] * cf[2] + P[at + s->n2 + 1] * cf[3];
    }
    double rho = v[0], uu = v[1];
    double Bp[4] = {0., v[5], v[6], v[7]};
    double Vc[4] = {0., v[2], v[3], v[4]};
    fs->ne = rho * c->Ne_unit;

    double VdotV = 0.;
    for (int p = 1; p < 4; p++)
        for (int q = 1; q < 4; q++)
            VdotV += gcov[p * 4 + q] * Vc[p] * Vc[q];
    double Vfac = sqrt(-1. / gcon[0] * (1. + fabs(VdotV)));
    double *U = fs->ucon;
    U[0] = -Vfac * gcon[0];
    for (int p = 1; p < 4; p++)
        U[p] = Vc[p] - Vfac * gcon[p];
    double Ucov[4], Bcov[4];
    lower(gcov, U, Ucov);
    double UdB = 0.;
    for (int p = 1; p < 4; p++)
        UdB += Ucov[p] * Bp[p];
    double *Bc = fs->bcon;
    Bc[0] = UdB;
    for (int p = 1; p < 4; p++)
        Bc[p] = (Bp[p] + U[p] * UdB) / U[0];
    lower(gcov, Bc, Bcov);
    fs->B = sqrt(Bc[0] * Bcov[0] + Bc[1] * Bcov[1] + Bc[2] * Bcov[2] + Bc[3] * Bcov[3]) * c->B_unit + tiny;
    double Bsq = (Bc[0] * Bcov[0] + Bc[1] * Bcov[1] + Bc[2] * Bcov[2] + Bc[3] * Bcov[3]);
    double beta_trans = 1.;
    fs->beta = uu * (4. / 3. - 1.) / (0.5 * (Bsq + tiny) * beta_trans);
    double b2 = pow(uu * (4. / 3. - 1.) / (0.5 * (Bsq + tiny) * beta_trans), 2);
    double trat = s->r_high * b2 / (1. + b2) + s->r_low / (1. + b2);
    double two_temp_gam = 0.5 * ((1. + 2. / 3. * (trat + 1.) / (trat + 2.)) + 4. / 3.);
    double Thetae_unit = (two_temp_gam - 1.) * (K_PMASS / K_EMASS) / (1. + trat);
    fs->thetae = ((uu) / (rho)) * Thetae_unit;
    if (fs->thetae < 0)
        fs->thetae = tiny;
    if (Bsq / rho > 1.0) {
        fs->ne = tiny;
        fs->thetae = tiny;
        fs->B = tiny;
        return 0;
    }
    return 1;
}

int port_fluid(const port_scene *s, const double X[4], double out[12])
{
    ray_ctx c;
    memset(&c, 0, sizeof c);
    c.s = s;
    double L = K_GGRAV * s->mbh / (K_CLIGHT * K_CLIGHT);
    double rho_unit = s->m_unit / pow(L, 3);
    c.B_unit = K_CLIGHT * sqrt(4. * K_PI * rho_unit);
    c.Ne_unit = rho_unit / (K_PMASS + K_EMASS);
    double gd[16], gu[16];
    port_metric_dd(s, X, gd);
    port_metric_uu(s, X, gu);
    fluid_state fs;
    int ok = fluid_params(&c, X, gd, gu, &fs);
    out[0] = fs.ne;
    out[1] = fs.thetae;
    out[2] = fs.B;
    out[3] = fs.beta;
    for (int q = 0; q < 4; q++) {
        out[4 + q] = fs.ucon[q];
        out[8 + q] = fs.bcon[q];
    }
    return ok;
}

/* ---- one transfer sample, radiative_transfer.c:49-119 ---- */
static int transfer(const ray_ctx *c, const double X[4], const double k[4], double dl,
                    const double *freqs, int nf, double *tau, double *I)
{
    double gd[16], gu[16];
    port_metric_dd(c->s, X, gd);
    port_metric_uu(c->s, X, gu);
    fluid_state fs;
    if (!fluid_params(c, X, gd, gu, &fs))
        return 0;
    double kd[4];
    lower(gd, k, kd);
    /* pitch_angle, radiative_transfer.c:32-47 (returns the cosine) */
    double pitch = 0.;
    if (fs.B != 0.) {
        const double *U = fs.ucon, *Bc = fs.bcon;
        double kk = fabs(kd[0] * U[0] + kd[1] * U[1] + kd[2] * U[2] + kd[3] * U[3]);
        pitch = (kd[0] * Bc[0] + kd[1] * Bc[1] + kd[2] * Bc[2] + kd[3] * Bc[3]) /
                (kk * fs.B / c->B_unit);
        if (fabs(pitch) > 1.)
            pitch /= fabs(pitch);
    }
    for (int f = 0; f < nf; f++) {
        double kuf[4], kdf[4];
        for (int q = 0; q < 4; q++)
            kuf[q] = k[q] * K_PLANCK * freqs[f] / (K_EMASS * K_CLIGHT * K_CLIGHT);
        lower(gd, kuf, kdf);
        /* freq_in_plasma_frame, radiative_transfer.c:17-29 */
        double nup = 0.;
        for (int q = 0; q < 4; q++)
            nup += fs.ucon[q] * kdf[q];
        nup *= -(K_EMASS * K_CLIGHT * K_CLIGHT) / K_PLANCK;
        if (nup <= 0.0)
            nup = 1.0;
        double nup2 = nup * nup;
        double j, an;
        if (c->s->emission == 1) { /* the kappa fits in emission_coeff's place */
            j = port_j_kappa(nup, fs.ne, fs.thetae, fs.B, pitch);
            an = port_a_kappa(nup, fs.ne, fs.thetae, fs.B, pitch);
        } else {
            j = port_j_thsynch(fs.B, pitch, fs.thetae, nup, fs.ne);
            an = port_a_th(j, nup, fs.thetae);
        }
        double dlf = dl * c->Rg / (freqs[f]);
        double dtau = (nup * an * dlf);
        tau[f] += dtau;
        double dI = (j / nup2) * exp(-tau[f]) * dlf;
        if (tau[f] < log(1000.) && !(tau[f] < 0.0))
            I[f] += dI;
    }
    return 1;
}

/* one per-step record, the layout of raptor_gpu_trace_ray */
static void record(double *rec, int cap, int steps, const double ph[8], double dl, double tau0, double I0,
                   int turns, int event, int stop)
{
    if (!rec || steps >= cap)
        return;
    double *r = rec + (size_t)steps * 16;
    for (int i = 0; i < 8; i++)
        r[i] = ph[i];
    r[8] = dl;
    r[9] = tau0;
    r[10] = I0;
    r[11] = steps;
    r[12] = turns;
    r[13] = event;
    r[14] = stop;
    r[15] = 0.;
}

/* ---- the per-pixel loop, integrator.c:149-289 ---- */
static void trace(const ray_ctx *c, int x, int y, const double *freqs, int nf, double *I,
                  port_ray_stats *st, double *rec, int cap)
{
    const port_scene *s = c->s;
    double tau[64];
    for (int f = 0; f < nf; f++) {
        tau[f] = 0.;
        I[f] = 0.;
    }
    double alpha, beta;
    if (s->camera == 1) {
        /* LOG_IMPACT_CAM, integrator.c:192-198 */
        double r_i = exp(log(20.) * (double)(x + 0.5) / ((double)s->width)) - 1.;
        double theta_i = 2.0 * K_PI * (double)(y + 0.5) / ((double)s->height);
        alpha = r_i * cos(theta_i);
        beta = r_i * sin(theta_i);
    } else {
        /* LINEAR_IMPACT_CAM, integrator.c:187-190 */
        double stepx = s->cam_size_x / (double)s->width;
        double stepy = s->cam_size_y / (double)s->height;
        alpha = -s->cam_size_x * 0.5 + (x + 0.5) * stepx;
        beta = -s->cam_size_y * 0.5 + (y + 0.5) * stepy;
    }
    double ph[8];
    FLOP_SNAP(f_init);
    init_photon(c, alpha, beta, ph);
    double r = exp(ph[1]);
    FLOP_ADD(0, f_init);
    int steps = 0, turns = 0, stop = 0, samples = 0, calls = 0, reason = 0;
    double thdot_prev = 0.;
    record(rec, cap, 0, ph, 0., tau[0], I[0], 0, 0, 0);
    while (r < K_CUTOFF_OUTER && r > c->cutoff_inner && steps < K_MAX_STEPS && !stop) {
        FLOP_SNAP(f_step);
        if (thdot_prev * ph[6] < 0. && steps > 2)
            turns += 1;
        thdot_prev = ph[6];
        if ((beta < 0. && turns > K_MAX_ORDER) || (beta > 0. && turns > (K_MAX_ORDER + 1)))
            stop = 1;
        double dl = step_size(s->stepsize, ph, ph + 4);
        double adl = fabs(dl);
        if (s->integrator == 2)
            step_rk2(s, ph, dl);
        else
            step_rk4(s, ph, dl);
        if (ph[1] > c->stopx1 && ph[5] < 0) {
            reason = 2;
            steps++;
            FLOP_ADD(1, f_step);
            record(rec, cap, steps, ph, dl, tau[0], I[0], turns, 3, stop);
            break;
        }
        r = exp(ph[1]);
        FLOP_ADD(1, f_step);
        int event = 0;
        if (ph[1] < c->stopx1 && ph[1] > s->startx1 && ph[2] > s->startx2 && ph[2] < c->stopx2) {
            calls++;
            FLOP_SNAP(f_rt);
            int ok = transfer(c, ph, ph + 4, adl, freqs, nf, tau, I);
            FLOP_ADD(ok ? 3 : 2, f_rt);
            samples += ok;
            event = ok ? 2 : 1;
        }
        record(rec, cap, steps + 1, ph, dl, tau[0], I[0], turns, event, stop);
        FLOP_SNAP(f_tail);
        r = exp(ph[1]);
        steps = steps + 1;
        FLOP_ADD(1, f_tail);
    }
    if (!reason) {
        if (!(r == r))
            reason = 6;
        else if (r <= c->cutoff_inner)
            reason = 1;
        else if (r >= K_CUTOFF_OUTER)
            reason = 3;
        else if (stop)
            reason = 5;
        else
            reason = 4;
    }
    if (st) {
        /* steps counts RK steps taken (the escape break is after a step) */
        st->steps = steps;
        st->rt_samples = samples;
        st->rt_calls = calls;
        st->reason = reason;
        double g[16];
        port_metric_dd(s, ph, g);
        double kk = 0.;
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
                kk += g[i * 4 + j] * ph[4 + i] * ph[4 + j];
        st->kk = fabs(kk) / (ph[4] * ph[4]);
    }
}

static void make_ctx(const port_scene *s, ray_ctx *c)
{
    memset(c, 0, sizeof *c);
    c->s = s;
    c->stopx1 = s->startx1 + s->n1 * s->dx1;
    c->stopx2 = s->startx2 + s->n2 * s->dx2;
    /* set_constants, utilities.c:19-20; set_units, grmhd.c:17-33 */
    double Rh = (1. + sqrt(1. - s->a * s->a));
    c->cutoff_inner = Rh * (1. + K_HORIZON_MARG);
    double L = K_GGRAV * s->mbh / (K_CLIGHT * K_CLIGHT);
    double rho_unit = s->m_unit / pow(L, 3);
    c->B_unit = K_CLIGHT * sqrt(4. * K_PI * rho_unit);
    c->Ne_unit = rho_unit / (K_PMASS + K_EMASS);
    c->Rg = K_GGRAV * s->mbh / K_CLIGHT / K_CLIGHT;
    c->cam_x2 = port_camera_x2(s);
}

int port_trace_ray(const port_scene *s, int pixel, const double *freqs, int nfreq, int cap, double *records)
{
    if (nfreq < 1 || nfreq > 64 || pixel < 0 || pixel >= s->width * s->height)
        return -1;
    ray_ctx c;
    make_ctx(s, &c);
    double I[64];
    port_ray_stats st;
    trace(&c, pixel % s->width, pixel / s->width, freqs, nfreq, I, &st, records, cap);
    return st.steps + 1 < cap ? st.steps + 1 : cap;
}

int port_render(const port_scene *s, const int *pixels, int n, const double *freqs, int nfreq,
                double *out, port_ray_stats *stats, int nthreads)
{
    if (nfreq < 1 || nfreq > 64)
        return -1;
    ray_ctx c;
    make_ctx(s, &c);
    double nu3[64];
    for (int f = 0; f < nfreq; f++)
        nu3[f] = pow(freqs[f], 3.);
#ifdef _OPENMP
    if (nthreads <= 0)
        nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
#endif
    for (int k = 0; k < n; k++) {
        int pix = pixels[k];
        int yy = pix / s->width, xx = pix % s->width;
        double I[64];
        trace(&c, xx, yy, freqs, nfreq, I, stats ? &stats[k] : NULL, NULL, 0);
        if (s->camera == 1) {
            /* core.c:123-133 */
            double r_grav = K_GGRAV * s->mbh / K_CLIGHT / K_CLIGHT;
            double r_i = exp(log(20.) * (double)(xx + 0.5) / (double)s->width) - 1.;
            double d_r = r_grav * (r_i + 1.) * log(20.) / (double)s->width;
            double d_theta = r_grav * 2. * K_PI / (double)s->height;
            for (int f = 0; f < nfreq; f++)
                out[(size_t)k * nfreq + f] =
                    I[f] * nu3[f] * r_i * d_r * d_theta / (K_SOURCE_DIST * K_SOURCE_DIST);
        } else {
            for (int f = 0; f < nfreq; f++)
                out[(size_t)k * nfreq + f] = I[f] * nu3[f];
        }
    }
    return 0;
}
