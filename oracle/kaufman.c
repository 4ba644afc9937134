/*
 * kaufman.c -- exact partition function of the 2D Ising model on an L x L
 * torus (periodic in both directions, J = 1, no field), in FP64.
 *
 * TEST INFRASTRUCTURE ONLY (the statistical oracle).  The reference has no
 * exact solution; this restates the published formula of B. Kaufman,
 * Phys. Rev. 76, 1232 (1949), in the form given by A. E. Ferdinand and
 * M. E. Fisher, Phys. Rev. 185, 832 (1969):
 *
 *   Z = 1/2 (2 sinh 2K)^(mn/2) (Z1 + Z2 + Z3 + Z4),
 *   Z1 = prod_{r<n} 2 cosh(m g_{2r+1}/2),  Z2 = prod_{r<n} 2 sinh(m g_{2r+1}/2),
 *   Z3 = prod_{r<n} 2 cosh(m g_{2r}/2),    Z4 = prod_{r<n} 2 sinh(m g_{2r}/2),
 *   cosh g_k = cosh 2K coth 2K - cos(pi k / n)   (k >= 1, g_k > 0),
 *   g_0 = 2K + ln tanh K                          (negative above K_c).
 *
 * Everything is evaluated in the log domain (products of up to 2L cosh/sinh
 * factors overflow FP64 for L >= 128), with the sign of Z4 carried
 * separately.  <E> = -d lnZ / dK is differentiated analytically; the heat
 * capacity C = K^2 d^2 lnZ / dK^2 is the central difference of <E>.
 */
#include <math.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static double log2cosh(double x) { x = fabs(x); return x + log1p(exp(-2.0 * x)); }
/* log |2 sinh x| */
static double log2sinh(double x) {
    x = fabs(x);
    if (x < 1e-3) return log(2.0 * x) + log1p(x * x / 6.0);
    return x + log(-expm1(-2.0 * x));
}

/* lnZ and dlnZ/dK for an m x n torus at coupling K */
static void kaufman_eval(int m, int n, double K, double* lnz, double* dlnz) {
    double c2 = cosh(2 * K), s2 = sinh(2 * K), coth2 = c2 / s2;
    double base = c2 * coth2;
    double dbase = 2 * c2 * (1 - 1 / (s2 * s2));
    double l[4] = {0, 0, 0, 0}, d[4] = {0, 0, 0, 0};
    int sign4 = 1;
    for (int r = 0; r < n; ++r) {
        for (int par = 0; par < 2; ++par) {
            int k = 2 * r + (par ? 1 : 0);
            double g, dg;
            if (k == 0) {
                g = 2 * K + log(tanh(K));
                dg = 2 + 2 / s2;
            } else {
                double ch = base - cos(M_PI * k / n);
                g = acosh(ch);
                dg = dbase / sinh(g);
            }
            double x = 0.5 * m * g, dx = 0.5 * m * dg;
            int ic = par ? 0 : 2, is = par ? 1 : 3;
            l[ic] += log2cosh(x);
            d[ic] += dx * tanh(x);
            l[is] += log2sinh(x);
            d[is] += dx / tanh(x);
            if (is == 3 && x < 0) sign4 = -sign4;
        }
    }
    double mx = l[0];
    for (int i = 1; i < 4; ++i) if (l[i] > mx) mx = l[i];
    double sum = 0, dsum = 0;
    for (int i = 0; i < 4; ++i) {
        if (!isfinite(l[i])) continue; /* Z4 = 0 exactly at K_c */
        double w = exp(l[i] - mx) * (i == 3 ? sign4 : 1);
        sum += w;
        dsum += w * d[i];
    }
    double N = (double)m * n;
    *lnz = -log(2.0) + 0.5 * N * log(2 * s2) + mx + log(sum);
    *dlnz = N * coth2 + dsum / sum;
}

/* lnZ, <E> and C (whole lattice, not per site) of the L x L torus at beta */
void or_kaufman(int L, double beta, double* lnZ, double* E, double* C) {
    double lz, dz;
    if (beta <= 0) {
        *lnZ = (double)L * L * log(2.0);
        *E = 0;
        *C = 0;
        return;
    }
    kaufman_eval(L, L, beta, &lz, &dz);
    *lnZ = lz;
    *E = -dz;
    double h = 1e-5 * (beta > 1e-2 ? beta : 1e-2), a, b, u, v;
    kaufman_eval(L, L, beta + h, &u, &a);
    kaufman_eval(L, L, beta - h, &v, &b);
    *C = beta * beta * (a - b) / (2 * h);
}
