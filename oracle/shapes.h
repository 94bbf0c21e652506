/* Synthetic bispectrum shapes shared by the CPU oracle and the in-place
 * reference build (test infrastructure only).
 *
 * The reference evaluates a shape through a per-point callback
 * (calculate_3D_bispectrum, calculate_mode_3D.c:266-281).  Here a shape is a
 * plain description that both CPU checkers and the CUDA kernels evaluate with
 * the same formula:
 *
 *   kind 0, separable:  S(l1,l2,l3) = sum_t (1/6) sum_{perm s} f_t(l_s1) g_t(l_s2) h_t(l_s3)
 *                       with f,g,h tabulated over l = 0..lmax ([T][3][lmax+1]).
 *   kind 1, Gaussian bump: L = l1+l2+l3,
 *                       S = exp(-((l1/L-c1)^2 + (l2/L-c2)^2 + (l3/L-c3)^2) / (2 sigma^2)),
 *                       evaluated at the tetrapyd point as given (l1<=l2<=l3).
 */
#ifndef MODAL_ORACLE_SHAPES_H
#define MODAL_ORACLE_SHAPES_H
#include <math.h>

typedef struct {
    int kind;            /* 0 separable table, 1 Gaussian bump */
    int nterms;          /* kind 0: number of separable terms T */
    int lmax;            /* kind 0: tables hold l = 0..lmax */
    const double *tab;   /* kind 0: [T][3][lmax+1] */
    double c1, c2, c3;   /* kind 1: centre on the simplex */
    double sigma;        /* kind 1: width */
} orc_shape;

static inline double orc_shape_eval(const orc_shape *s, int l1, int l2, int l3)
{
    if (s->kind == 0) {
        const int stride = s->lmax + 1;
        double acc = 0.0;
        for (int t = 0; t < s->nterms; t++) {
            const double *f = s->tab + (long)t * 3 * stride;
            const double *g = f + stride;
            const double *h = g + stride;
            double v = f[l1] * g[l2] * h[l3] + f[l1] * g[l3] * h[l2]
                     + f[l2] * g[l1] * h[l3] + f[l2] * g[l3] * h[l1]
                     + f[l3] * g[l1] * h[l2] + f[l3] * g[l2] * h[l1];
            acc += v / 6.0;
        }
        return acc;
    } else {
        double L = (double)(l1 + l2 + l3);
        double x1 = l1 / L - s->c1, x2 = l2 / L - s->c2, x3 = l3 / L - s->c3;
        return exp(-(x1 * x1 + x2 * x2 + x3 * x3) / (2.0 * s->sigma * s->sigma));
    }
}
#endif
