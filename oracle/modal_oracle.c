/* modal_oracle.c -- CPU FP64 restatement of the Modal-CMB mode-space hot path.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg load this library, and only as a checker or
 * as the timed CPU baseline.  The CUDA library never calls it.
 *
 * Each function restates one reference routine (file:line in the Modal-CMB
 * sources) in plain C with the same arithmetic, so that outputs can be
 * compared element-wise with the CUDA path.  The restatement is itself pinned
 * against the reference sources compiled in place (oracle/_ref, see
 * oracle/Makefile) and against golden vectors under tests/golden/ that were
 * produced by that build.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>
#include "shapes.h"

#define ORC_PI 3.14159265358979323846

/* ------------------------------------------------------------------------ */
/* Gauss-Legendre nodes and weights.                                          */
/* Layout as asy() (gl_integration.c:46-168): nodes ascending on [-1,1],      */
/* symmetric pairs nodes[k-1] = -nodes[n-k], exact 0 for the middle node of  */
/* odd n (gl_integration.c:156-165).  The reference uses the Hale-Townsend    */
/* asymptotic method (QUADPTS, GPL-3+); this restatement instead runs Newton  */
/* in theta (x = cos theta) from Tricomi's initial guess, evaluating P_n by   */
/* the three-term recurrence written in differences D_l = P_l - P_{l-1} and   */
/* y = 1 - x = 2 sin^2(theta/2):                                              */
/*     D_{l+1} = (l D_l - (2l+1) y P_l) / (l+1),   P_{l+1} = P_l + D_{l+1},   */
/* which keeps full relative accuracy next to x = 1 where the endpoint        */
/* weights dominate the Gamma integrand.  Weight:                              */
/*     w = 2 sin^2(theta) / (n (P_{n-1} - x P_n))^2.                          */
/* Arithmetic in long double.                                                  */
/* ------------------------------------------------------------------------ */
static void gl_leg_diff(int n, long double th, long double *Pn, long double *Q)
{
    long double s = sinl(0.5L * th), y = 2.0L * s * s;
    long double P = 1.0L, D = 0.0L;
    for (int l = 0; l < n; l++) {
        long double Dn = (l * D - (2.0L * l + 1.0L) * y * P) / (l + 1.0L);
        P += Dn;
        D = Dn;
    }
    *Pn = P;
    *Q = -D + y * P; /* P_{n-1} - x P_n */
}

int orc_gl_nodes(int n, double *nodes, double *weights)
{
    if (n < 1) return 1;
    const long double pi = 3.141592653589793238462643383279502884L;
    const int half = n / 2;
    for (int k = 1; k <= half; k++) {
        long double th = pi * (4.0L * k - 1.0L) / (4.0L * n + 2.0L);
        long double x0 = (1.0L - (n - 1.0L) / (8.0L * n * n * n)) * cosl(th);
        th = acosl(x0);
        long double Pn, Q;
        for (int it = 0; it < 100; it++) {
            gl_leg_diff(n, th, &Pn, &Q);
            long double dth = Pn * sinl(th) / (n * Q);
            th += dth;
            if (fabsl(dth) <= 1e-19L * th) break;
        }
        gl_leg_diff(n, th, &Pn, &Q);
        long double st = sinl(th);
        long double w = 2.0L * st * st / ((long double)n * n * Q * Q);
        nodes[n - k] = (double)cosl(th);
        nodes[k - 1] = -(double)cosl(th);
        weights[n - k] = (double)w;
        weights[k - 1] = (double)w;
    }
    if (n & 1) {
        long double Pn, Q;
        gl_leg_diff(n, pi / 2.0L, &Pn, &Q);
        nodes[half] = 0.0;
        weights[half] = (double)(2.0L / ((long double)n * n * Q * Q));
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* gl_Pl[k][l] = (2l+1)^{2/3} P_l(mu_k), l = 0..lmax                           */
/* (orthogonalisation_late.c:47-54).  P_l as GSL's gsl_sf_legendre_Pl: the   */
/* upward recurrence p_l = (x(2l-1)p_{l-1} - (l-1)p_{l-2})/l from P_0, P_1,  */
/* with P_2 = (3x^2-1)/2 returned in closed form.  One pass per mu gives the  */
/* same values GSL computes per (l, mu) call.                                  */
/* ------------------------------------------------------------------------ */
int orc_legendre_table(int nmu, int lmax, const double *mu, double *out /*[nmu][lmax+1]*/)
{
    #pragma omp parallel for schedule(static)
    for (int k = 0; k < nmu; k++) {
        const double x = mu[k];
        double *row = out + (long)k * (lmax + 1);
        double pm2 = 1.0, pm1 = x;
        for (int l = 0; l <= lmax; l++) {
            double p;
            if (l == 0) p = 1.0;
            else if (l == 1) p = x;
            else {
                double pr = (x * (2 * l - 1) * pm1 - (l - 1) * pm2) / l;
                pm2 = pm1; pm1 = pr;
                if (l == 2) p = 0.5 * (3.0 * x * x - 1.0);
                else if (x == 1.0) p = 1.0;
                else if (x == -1.0) p = (l & 1) ? -1.0 : 1.0;
                else p = pr;
            }
            row[l] = pow(2e0 * l + 1e0, 2e0 / 3e0) * p;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Shifted Legendre basis q_j(v_i) = P_j(2(v_i-min)/(max-min) - 1)            */
/* (basis_functions.c:88-107), out[size][pmax+1].                              */
/* ------------------------------------------------------------------------ */
int orc_basis_legendre(int size, int pmax, double min, double max, const double *values, double *out)
{
    for (int i = 0; i < size; i++) {
        double *a = out + (long)i * (pmax + 1);
        double x = (values[i] - min) / (max - min);
        a[0] = 1e0;
        if (pmax > 0) a[1] = 2e0 * x - 1e0;
        for (int j = 2; j <= pmax; j++)
            a[j] = ((2e0 * j - 1e0) * a[1] * a[j - 1] - (j - 1e0) * a[j - 2]) / (1e0 * j);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* l-contraction M[i][j][s] = sum_{l=lmin}^{lmax} gl_Pl[s][l] q_i(l) q_j(l)   */
/* (orthogonalisation_late.c:99-129, all P^2 (i,j) as ortho_late_mpi.c:170).  */
/* basis[L][P] with L = lmax-lmin+1; out[P][P][nmu].                           */
/* ------------------------------------------------------------------------ */
int orc_mij(int nmu, int lmin, int lmax, int P, const double *gl_pl, const double *basis, double *out)
{
    const int L = lmax - lmin + 1;
    #pragma omp parallel for collapse(2) schedule(static)
    for (int i = 0; i < P; i++)
        for (int j = 0; j < P; j++) {
            double *vec = malloc(sizeof(double) * (size_t)L);
            for (int l = 0; l < L; l++) vec[l] = basis[(long)l * P + i] * basis[(long)l * P + j];
            for (int s = 0; s < nmu; s++) {
                const double *row = gl_pl + (long)s * (lmax + 1);
                double sum = 0e0;
                for (int l = lmin; l <= lmax; l++) sum += row[l] * vec[l - lmin];
                out[((long)i * P + j) * nmu + s] = sum;
            }
            free(vec);
        }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* gamma_mn = sum_k w_k/(48 pi) sum of the six products                       */
/* (calculate_orthol, orthogonalisation_late.c:239-336, TTT part :283-295).   */
/* ------------------------------------------------------------------------ */
static double orthol_pair(int P, int nmu, const double *M, const double *w, const int *tm, const int *tn)
{
#define MM(a, b) (M + ((long)(a) * P + (b)) * nmu)
    const double *a11 = MM(tm[0], tn[0]), *a22 = MM(tm[1], tn[1]), *a33 = MM(tm[2], tn[2]);
    const double *a21 = MM(tm[1], tn[0]), *a32 = MM(tm[2], tn[1]), *a13 = MM(tm[0], tn[2]);
    const double *a31 = MM(tm[2], tn[0]), *a12 = MM(tm[0], tn[1]), *a23 = MM(tm[1], tn[2]);
#undef MM
    double r = 0e0;
    for (int i = 0; i < nmu; i++) {
        double wgt1 = w[i] / (48e0 * ORC_PI);
        double s1 = a11[i] * a22[i] * a33[i];
        double s2 = a21[i] * a32[i] * a13[i];
        double s3 = a31[i] * a12[i] * a23[i];
        double s4 = a31[i] * a22[i] * a13[i];
        double s5 = a21[i] * a12[i] * a33[i];
        double s6 = a11[i] * a32[i] * a23[i];
        double sum = s1 + s2 + s3 + s4 + s5 + s6;
        r += wgt1 * sum;
    }
    return r;
}

int orc_orthol_pair(int P, int nmu, const double *M, const double *w, const int *triples, int m, int n, double *result)
{
    result[0] = orthol_pair(P, nmu, M, w, triples + 3 * m, triples + 3 * n);
    return 0;
}

/* Full symmetric Gamma[N][N] from the upper triangle (ortho_late_mpi.c:231-363). */
int orc_gamma(int N, const int *triples, int P, int nmu, const double *M, const double *w, int nthreads, double *out)
{
    if (nthreads > 0) omp_set_num_threads(nthreads);
    #pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < N; i++)
        for (int j = i; j < N; j++) {
            double g = orthol_pair(P, nmu, M, w, triples + 3 * i, triples + 3 * j);
            out[(long)i * N + j] = g;
            out[(long)j * N + i] = g;
        }
    return 0;
}

/* Polarised Gamma, results[1..3] of calculate_orthol with do_polarisation
 * (orthogonalisation_late.c:293-320).  M tables as Mij_T / Mij_E
 * [P][P][nmu]; mode triples in the find_perm_late_XXX conventions:
 * tte[n] = (T, T, E), tee[n] = (T, E, E), eee[n] = (E, E, E).
 *   TTE: sum_k w_k/(16 pi) (MT[a0][b0] MT[a1][b1] + MT[a1][b0] MT[a0][b1]) ME[a2][b2]
 *   TEE: sum_k w_k/(16 pi) MT[a0][b0] (ME[a1][b1] ME[a2][b2] + ME[a2][b1] ME[a1][b2])
 *   EEE: as TTT with ME and w_k/(48 pi).
 * Any output may be NULL. */
int orc_gamma_pol(int N, const int *tte, const int *tee, const int *eee, int PT, int PE, int nmu, const double *MT,
                  const double *ME, const double *w, double *g_tte, double *g_tee, double *g_eee)
{
#define ORC_MT(a, b, k) MT[((long)(a) * PT + (b)) * nmu + (k)]
#define ORC_ME(a, b, k) ME[((long)(a) * PE + (b)) * nmu + (k)]
    #pragma omp parallel for schedule(dynamic, 4)
    for (int m = 0; m < N; m++)
        for (int n = m; n < N; n++) {
            double r2 = 0.0, r3 = 0.0;
            const int *a = tte + 3 * m, *b = tte + 3 * n, *c = tee + 3 * m, *d = tee + 3 * n;
            for (int k = 0; k < nmu; k++) {
                const double wgt2 = w[k] / (16e0 * ORC_PI);
                double s1 = ORC_MT(a[0], b[0], k) * ORC_MT(a[1], b[1], k) * ORC_ME(a[2], b[2], k);
                double s2 = ORC_MT(a[1], b[0], k) * ORC_MT(a[0], b[1], k) * ORC_ME(a[2], b[2], k);
                r2 += wgt2 * (s1 + s2);
                s1 = ORC_MT(c[0], d[0], k) * ORC_ME(c[1], d[1], k) * ORC_ME(c[2], d[2], k);
                s2 = ORC_MT(c[0], d[0], k) * ORC_ME(c[2], d[1], k) * ORC_ME(c[1], d[2], k);
                r3 += wgt2 * (s1 + s2);
            }
            if (g_tte) g_tte[(long)m * N + n] = g_tte[(long)n * N + m] = r2;
            if (g_tee) g_tee[(long)m * N + n] = g_tee[(long)n * N + m] = r3;
            if (g_eee) {
                double g = orthol_pair(PE, nmu, ME, w, eee + 3 * m, eee + 3 * n);
                g_eee[(long)m * N + n] = g_eee[(long)n * N + m] = g;
            }
        }
#undef ORC_MT
#undef ORC_ME
    return 0;
}

/* Gamma for the first `npairs` upper-triangle pairs (row-major order) only,
 * for bounded CPU timing samples; returns the number of pairs done. */
long orc_gamma_sample(int N, const int *triples, int P, int nmu, const double *M, const double *w, int nthreads,
                      long npairs, double *out_pairs)
{
    long total = (long)N * (N + 1) / 2;
    if (npairs <= 0 || npairs > total) npairs = total;
    if (nthreads > 0) omp_set_num_threads(nthreads);
    #pragma omp parallel for schedule(static)
    for (long p = 0; p < npairs; p++) {
        /* invert p -> (i,j), i<=j, row-major over the upper triangle */
        long i = (long)((2.0 * N + 1 - sqrt((2.0 * N + 1) * (2.0 * N + 1) - 8.0 * p)) / 2.0);
        if (i < 0) i = 0;
        while (i > 0 && i * N - i * (i - 1) / 2 > p) i--;
        while ((i + 1) * N - (i + 1) * i / 2 <= p) i++;
        long j = i + (p - (i * N - i * (i - 1) / 2));
        out_pairs[p] = orthol_pair(P, nmu, M, w, triples + 3 * i, triples + 3 * j);
    }
    return npairs;
}

/* ------------------------------------------------------------------------ */
/* Asymptotic geometric factor h~^2 (calculate_geometric.c:59-92).            */
/* ------------------------------------------------------------------------ */
double orc_geometric(int l1, int l2, int l3)
{
    if (((l1 + l2 + l3) % 2) == 0 && l1 + l2 >= l3 && l2 + l3 >= l1 && l3 + l1 >= l2) {
        double s1 = l1 + l2 + l3 + 1.0;
        double s3 = l1 + l2 + l3 + 1.0 / 3.0;
        double s6 = l1 + l2 + l3 + 1.0 / 6.0;
        double s13 = l2 + l3 - l1 + 1.0 / 3.0;
        double s23 = l3 + l1 - l2 + 1.0 / 3.0;
        double s33 = l1 + l2 - l3 + 1.0 / 3.0;
        double s16 = l2 + l3 - l1 + 1.0 / 6.0;
        double s26 = l3 + l1 - l2 + 1.0 / 6.0;
        double s36 = l1 + l2 - l3 + 1.0 / 6.0;
        double fact = (1.0 / ORC_PI) * (1.0 / ORC_PI) / 2.0;
        double p1 = fact * ((2.0 * l1 + 1.0) * (2.0 * l2 + 1.0) * (2.0 * l3 + 1.0)) / s1;
        double p2 = s3 / (s13 * s23 * s33);
        double p3 = sqrt(s16 * s26 * s36 / s6);
        return p1 * p2 * p3;
    }
    return 0.0;
}

/* permsix (fixed_data.c:4244-4254): distinct orderings of (i,j,k). */
double orc_permsix(int i, int j, int k)
{
    if (i == k && i == j) return 1.0;
    if (i == j || j == k || i == k) return 3.0;
    return 6.0;
}

/* ------------------------------------------------------------------------ */
/* Tetrapyd walk (tetrapyd_tools.c:104-142): i<=j<=k<=lmax, k<=i+j, i+j+k    */
/* even, k stepping by 2, starting from check_ijk_min_XXX (:144-180).         */
/* ------------------------------------------------------------------------ */
int orc_tetrapyd_next(int lmax, int *i1, int *j1, int *k1)
{
    int i = *i1, j = *j1, k = *k1, test = 1;
    if (i % 2 + j == lmax) { i++; j = i; k = j + i % 2; }
    else if (k + 2 > lmax || k >= i + j) { j++; k = j + i % 2; }
    else k += 2;
    if (i + j + k + 1 >= 3 * lmax) {
        test = 0;
        if (lmax % 2 == 0) { i = lmax; j = lmax; k = lmax; }
        else { i = lmax - 1; j = lmax; k = lmax; }
    }
    *i1 = i; *j1 = j; *k1 = k;
    return test;
}

void orc_tetrapyd_start(int lmin, int *i, int *j, int *k)
{
    int i0 = *i < lmin ? lmin : *i, j0 = *j < lmin ? lmin : *j, k0 = *k < lmin ? lmin : *k, n;
    if (i0 > j0) { n = j0; j0 = i0; i0 = n; }
    if (j0 > k0) { n = j0; j0 = k0; k0 = n; if (i0 > j0) { n = j0; j0 = i0; i0 = n; } }
    if (i0 + j0 < k0) k0 = i0 + j0;
    else if ((i0 + j0 + k0) % 2 == 1) k0 = k0 + 1;
    *i = i0; *j = j0; *k = k0;
}

/* Number of points the reference's decomposition assigns
 * (decompose_tetrapyd_XXX, tetrapyd_tools.c:31-51). */
long orc_tetrapyd_count(int lmin, int lmax)
{
    int i = lmin, j = lmin, k = lmin;
    orc_tetrapyd_start(lmin, &i, &j, &k);
    long count;
    long countmax = (long)lmax * lmax * lmax + 1;
    for (count = 1; count < countmax; count++)
        if (!orc_tetrapyd_next(lmax, &i, &j, &k)) break;
    return count + 1;
}

/* ------------------------------------------------------------------------ */
/* Projection (calculate_mode_3D, calculate_mode_3D.c:217-264):              */
/* beta_r = sum over the walk of get_weight(i,j,k) S(i,j,k) w_i w_j w_k     */
/*          * plijk_TTT(r,i,j,k)                                              */
/* get_weight = permsix h~^2 prod (2l+1)^{-1/3} (:283-290);                   */
/* w_l = (2l+1)^{1/6}/sqrt(C_l + N_l/b_l^2), w_0 = w_1 = 0 (:53-62);          */
/* plijk_TTT (orthogonalisation_late.c:620-644) with basis index l - lmin.    */
/* cl[l] holds C_l + N_l/b_l^2.  Walk points split over threads as          */
/* decompose_tetrapyd_XXX does (equal contiguous counts).                     */
/* `max_points` > 0 truncates each thread's block (timing samples).           */
/* ------------------------------------------------------------------------ */
static double plijk(const double *basis, int P, const int *tr, int lmin, int lmax, int l1, int l2, int l3)
{
    if (l1 < lmin || l1 > lmax || l2 < lmin || l2 > lmax || l3 < lmin || l3 > lmax) return 0e0;
    const double *bi = basis + (long)(l1 - lmin) * P, *bj = basis + (long)(l2 - lmin) * P, *bk = basis + (long)(l3 - lmin) * P;
    const int p1 = tr[0], p2 = tr[1], p3 = tr[2];
    double b1 = bi[p1] * bj[p2] * bk[p3];
    double b2 = bi[p2] * bj[p3] * bk[p1];
    double b3 = bi[p3] * bj[p1] * bk[p2];
    double b4 = bi[p3] * bj[p2] * bk[p1];
    double b5 = bi[p2] * bj[p1] * bk[p3];
    double b6 = bi[p1] * bj[p3] * bk[p2];
    return (b1 + b2 + b3 + b4 + b5 + b6) / (6e0);
}

double orc_plijk(const double *basis, int P, const int *triples, int lmin, int lmax, int r, int l1, int l2, int l3)
{
    return plijk(basis, P, triples + 3 * r, lmin, lmax, l1, l2, l3);
}

static void weights_l(int lmax, const double *cl, double *wl)
{
    wl[0] = 0e0;
    if (lmax >= 1) wl[1] = 0e0;
    for (int i = 2; i <= lmax; i++) wl[i] = pow(2.0 * i + 1.0, 1.0 / 6.0) / sqrt(cl[i]);
}

int orc_project(int lmin, int lmax, int P, const double *basis, int N, const int *triples, const double *cl,
                int kind, int nterms, const double *tab, double c1, double c2, double c3, double sigma,
                int nthreads, long max_points, double *beta)
{
    orc_shape sh = {kind, nterms, lmax, tab, c1, c2, c3, sigma};
    double *wl = malloc(sizeof(double) * (size_t)(lmax + 1));
    weights_l(lmax, cl, wl);
    long count = orc_tetrapyd_count(lmin, lmax);
    if (nthreads <= 0) nthreads = omp_get_max_threads();
    /* block starts as decompose_tetrapyd_XXX (one rank) */
    long *loops = malloc(sizeof(long) * (size_t)nthreads);
    int *start = malloc(sizeof(int) * 3 * (size_t)nthreads);
    {
        long size = count / nthreads, extra = count % nthreads;
        for (int t = 0; t < nthreads; t++) loops[t] = size + (t < extra ? 1 : 0);
        int i = lmin, j = lmin, k = lmin;
        orc_tetrapyd_start(lmin, &i, &j, &k);
        for (int t = 0; t < nthreads; t++) {
            start[3 * t] = i; start[3 * t + 1] = j; start[3 * t + 2] = k;
            for (long s = 0; s < loops[t]; s++) orc_tetrapyd_next(lmax, &i, &j, &k);
        }
    }
    for (int r = 0; r < N; r++) beta[r] = 0e0;
    omp_set_num_threads(nthreads);
    #pragma omp parallel
    {
        int t = omp_get_thread_num();
        double *priv = calloc((size_t)N, sizeof(double));
        int i = start[3 * t], j = start[3 * t + 1], k = start[3 * t + 2];
        long nl = loops[t];
        if (max_points > 0 && nl > max_points) nl = max_points;
        for (long n = 0; n < nl; n++) {
            double gw = orc_permsix(i, j, k) * orc_geometric(i, j, k) * pow(2.0 * i + 1.0, -1.0 / 3.0)
                      * pow(2.0 * j + 1.0, -1.0 / 3.0) * pow(2.0 * k + 1.0, -1.0 / 3.0);
            double x = gw * orc_shape_eval(&sh, i, j, k) * wl[i] * wl[j] * wl[k];
            for (int r = 0; r < N; r++) priv[r] += x * plijk(basis, P, triples + 3 * r, lmin, lmax, i, j, k);
            orc_tetrapyd_next(lmax, &i, &j, &k);
        }
        #pragma omp critical
        for (int r = 0; r < N; r++) beta[r] += priv[r];
        free(priv);
    }
    free(loops); free(start); free(wl);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Orthogonalisation, Cholesky branch (ortho_late_mpi.c:759-773, 806-843):    */
/*   norm_i = sqrt(gamma_ii); ghat = gamma_ij/(norm_i norm_j);               */
/*   ghat = L L^T (gsl_linalg_cholesky_decomp);                               */
/*   orthol[i][j] = norm_i L_ij (i>=j), 0 above;                             */
/*   lambdal[i][j] = ((L^T)^{-1})[j][i] / norm_j (gsl_linalg_LU_invert of the */
/*   upper factor with the identity permutation).                             */
/* Returns 0, or 1 + the failing pivot row when ghat is not positive          */
/* definite (GSL reports GSL_EDOM there).                                     */
/* ------------------------------------------------------------------------ */
long orc_ortho_cholesky(int N, const double *gamma, double *orthol, double *lambdal)
{
    double *norm = malloc(sizeof(double) * (size_t)N);
    double *A = malloc(sizeof(double) * (size_t)N * N);
    for (int i = 0; i < N; i++) norm[i] = sqrt(gamma[(long)i * N + i]);
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) A[(long)i * N + j] = gamma[(long)i * N + j] / (norm[i] * norm[j]);
    /* left-looking Cholesky, lower triangle */
    for (int j = 0; j < N; j++) {
        double d = A[(long)j * N + j];
        for (int k = 0; k < j; k++) d -= A[(long)j * N + k] * A[(long)j * N + k];
        if (!(d > 0.0)) { free(norm); free(A); return 1 + (long)j; }
        double ljj = sqrt(d);
        A[(long)j * N + j] = ljj;
        #pragma omp parallel for schedule(static)
        for (int i = j + 1; i < N; i++) {
            double s = A[(long)i * N + j];
            for (int k = 0; k < j; k++) s -= A[(long)i * N + k] * A[(long)j * N + k];
            A[(long)i * N + j] = s / ljj;
        }
    }
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) orthol[(long)i * N + j] = (i >= j) ? norm[i] * A[(long)i * N + j] : 0e0;
    /* inverse of U = L^T by back substitution, column by column:
       Uinv[r][c] for r <= c; lambdal[i][j] = Uinv[j][i] / norm[j]. */
    double *Uinv = calloc((size_t)N * N, sizeof(double));
    #pragma omp parallel for schedule(dynamic, 8)
    for (int c = 0; c < N; c++) {
        for (int r = c; r >= 0; r--) {
            double s = (r == c) ? 1.0 : 0.0;
            for (int k = r + 1; k <= c; k++) s -= A[(long)k * N + r] * Uinv[(long)k * N + c]; /* U[r][k] = L[k][r] */
            Uinv[(long)r * N + c] = s / A[(long)r * N + r];
        }
    }
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) lambdal[(long)i * N + j] = Uinv[(long)j * N + i] / norm[j];
    free(Uinv); free(norm); free(A);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Alpha solve (eigenmodetoday_mpi.c:148-162, 286-316):                       */
/*   lambdainv = lower triangle of orthol; orthoinv = lambdal^T lambdal;      */
/*   alpha = orthoinv beta; modesR_i = sum_j lambdainv[j][i] alpha_j.         */
/* ------------------------------------------------------------------------ */
int orc_alpha(int N, const double *orthol, const double *lambdal, const double *beta, double *alpha, double *modesR)
{
    double *orthoinv = malloc(sizeof(double) * (size_t)N * N);
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) {
            double s = 0.0;
            for (int k = 0; k < N; k++) s += lambdal[(long)k * N + i] * lambdal[(long)k * N + j];
            orthoinv[(long)i * N + j] = s;
        }
    for (int i = 0; i < N; i++) {
        double s = 0.0;
        for (int j = 0; j < N; j++) s += orthoinv[(long)i * N + j] * beta[j];
        alpha[i] = s;
    }
    for (int i = 0; i < N; i++) {
        double x = 0.0;
        for (int j = 0; j < N; j++) x += (i <= j ? orthol[(long)j * N + i] : 0.0) * alpha[j];
        modesR[i] = x;
    }
    free(orthoinv);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Serial dense form (calculate_modes.c:6-79).                                */
/* modify_bispectrum: b[i][j][k] <- c_i c_j c_k h~^2(l) (1.55e-8)^2 b on even */
/* triangle triples of l = vec[index], else 0; c_i = beam_i / ((2l_i+1)^{1/6}  */
/* sqrt(beam_i^2 cl_i + noise_i)) when cl_i != 0 and vec_i != 0.               */
/* calculate_modes: beta_r = sum_{i<=j<=k<size, b != 0} m plijk(r,i,j,k) b,    */
/* m = 1, 3, 6 by coinciding indices; the index is used as l.                 */
/* ------------------------------------------------------------------------ */
int orc_modify_bispectrum(int size, const int *vec, const double *cl, const double *beam, const double *noise,
                          double *b)
{
    double *c = malloc(sizeof(double) * (size_t)size);
    for (int i = 0; i < size; i++) {
        c[i] = 0;
        if (cl[i] != 0 && vec[i] != 0)
            c[i] = beam[i] / (pow(2.0 * vec[i] + 1.0, 1.0 / 6.0) * sqrt(beam[i] * beam[i] * cl[i] + noise[i]));
    }
    for (int i = 0; i < size; i++)
        for (int j = 0; j < size; j++)
            for (int k = 0; k < size; k++) {
                int a = vec[i], bb = vec[j], cc = vec[k];
                double *v = b + ((long)i * size + j) * size + k;
                if (((a + bb + cc) % 2) == 0 && a + bb >= cc && bb + cc >= a && cc + a >= bb)
                    *v = c[i] * c[j] * c[k] * orc_geometric(a, bb, cc) * (*v * 1.55e-8 * 1.55e-8);
                else
                    *v = 0.0;
            }
    free(c);
    return 0;
}

int orc_calculate_modes(int lmin, int lmax, int P, const double *basis, int N, const int *triples, int size,
                        const double *b, double *beta)
{
    #pragma omp parallel for schedule(dynamic, 1)
    for (int r = 0; r < N; r++) {
        double result = 0.0;
        for (int i = 0; i < size; i++)
            for (int j = i; j < size; j++)
                for (int k = j; k < size; k++) {
                    double v = b[((long)i * size + j) * size + k];
                    if (v != 0.0) {
                        double f = (i == j && j == k) ? 1.0 : ((i == j || j == k) ? 3.0 : 6.0);
                        result += f * plijk(basis, P, triples + 3 * r, lmin, lmax, i, j, k) * v;
                    }
                }
        beta[r] = result;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Late x primordial transfer Gamma, default path of gamma_mpi.c:            */
/* init_gamma_glint + precompute_gammaMij_T + calculate_gamma_2d             */
/* (calculate_gamma.c:48-303, 512-555, 773-934).                             */
/* ------------------------------------------------------------------------ */

/* integrate_cubic_spline (calculate_gamma.c:845-934): the integral over
 * [x0, x_{n-1}] of the reference's cubic spline through (x, y). */
double orc_integrate_cubic_spline(const double *x, const double *y, int npts)
{
    if (npts < 2) return 0.0;
    double *X = malloc(sizeof(double) * (size_t)npts), *Y = malloc(sizeof(double) * (size_t)npts);
    double *a = calloc((size_t)npts, sizeof(double)), *b = calloc((size_t)npts, sizeof(double));
    double *c = calloc((size_t)npts, sizeof(double));
    for (int i = 0; i < npts; i++) { X[i] = x[i]; Y[i] = y[i]; }
    c[0] = X[1] - X[0];
    b[1] = (Y[1] - Y[0]) / c[0];
    for (int i = 1; i < npts - 1; i++) {
        c[i] = x[i + 1] - X[i];
        a[i] = 2.0 * (c[i - 1] + c[i]);
        b[i + 1] = (Y[i + 1] - Y[i]) / c[i];
        b[i] = b[i + 1] - b[i];
    }
    a[0] = -c[0];
    a[npts - 1] = -c[npts - 2];
    b[0] = 0.0;
    b[npts - 1] = 0.0;
    if (npts > 2) {
        b[0] = b[2] / (X[3] - X[1]) - b[1] / (X[2] - X[0]);
        b[npts - 1] = b[npts - 2] / (X[npts - 1] - X[npts - 3]) - b[npts - 3] / (X[npts - 2] - X[npts - 4]);
        b[0] = b[0] * c[0] * c[0] / (X[3] - X[0]);
        b[npts - 1] = -b[npts - 1] * c[npts - 2] * c[npts - 2] / (X[npts - 1] - X[npts - 4]);
    }
    for (int i = 1; i < npts; i++) {
        double h = c[i - 1] / a[i - 1];
        a[i] = a[i] - h * c[i - 1];
        b[i] = b[i] - h * b[i - 1];
    }
    b[npts - 1] = b[npts - 1] / a[npts - 1];
    for (int i = npts - 2; i >= 0; i--) b[i] = (b[i] - c[i] * b[i + 1]) / a[i];
    a[npts - 1] = (Y[npts - 1] - Y[npts - 2]) / c[npts - 2] + c[npts - 2] * (b[npts - 2] + 2.0 * b[npts - 1]);
    for (int i = 0; i < npts - 1; i++) {
        a[i] = (Y[i + 1] - Y[i]) / c[i] - c[i] * (b[i + 1] + 2.0 * b[i]);
        c[i] = (b[i + 1] - b[i]) / c[i];
        b[i] = 3.0 * b[i];
    }
    b[npts - 1] = 3.0 * b[npts - 1];
    c[npts - 1] = c[npts - 2];
    double in = 0.0;
    for (int i = 0; i < npts - 1; i++) {
        double d = x[i + 1] - x[i];
        in += d * (Y[i] + d * (a[i] / 2.0 + d * (b[i] / 3.0 + d * c[i] / 4.0)));
    }
    free(X); free(Y); free(a); free(b); free(c);
    return in;
}

/* qt[x][p][l]: raw transfer functions q~_p(l, x), l = 0..lmax; prim[Nprim][3];
 * cl[l] = C_l + N_l/b_l^2 (beam 1 folded in); mu, w: n_mu GL nodes (asy());
 * out[N][Nprim] = calculate_gamma_2d(m, n) for late mode m and primordial n. */
int orc_gamma_transfer(int lmin, int lmax, int P, const double *basis, int N, const int *triples, const double *cl,
                       int nmu, const double *mu, const double *w, int xsize, const double *xvec, int Pp,
                       const double *qt, int Nprim, const int *prim, double dphi, double *out)
{
    const int L = lmax - lmin + 1;
    double *ttw = malloc(sizeof(double) * (size_t)L);
    for (int i = 0; i < L; i++) {
        int l = lmin + i;
        ttw[i] = (l > 1) ? pow(2e0 * l + 1e0, 5e0 / 6e0) * (1.0 / sqrt(cl[l])) : 0e0;  /* :76-88, beam 1 */
    }
    /* gl_Pl[k][l] = P_l(mu_k), no (2l+1) factor here (:97-101) */
    double *pl = malloc(sizeof(double) * (size_t)nmu * (lmax + 1));
    #pragma omp parallel for
    for (int k = 0; k < nmu; k++) {
        double x = mu[k], pm2 = 1.0, pm1 = x;
        double *row = pl + (long)k * (lmax + 1);
        for (int l = 0; l <= lmax; l++) {
            double p;
            if (l == 0) p = 1.0;
            else if (l == 1) p = x;
            else {
                double pr = (x * (2 * l - 1) * pm1 - (l - 1) * pm2) / l;
                pm2 = pm1; pm1 = pr;
                p = (l == 2) ? 0.5 * (3.0 * x * x - 1.0) : (x == 1.0 ? 1.0 : (x == -1.0 ? ((l & 1) ? -1.0 : 1.0) : pr));
            }
            row[l] = p;
        }
    }
    /* M[p][q][x][k] = sum_l gl_Pl[k][l+lmin] qtilde_T[x][p][l] basis_T[q][l] (:254-303) */
    double *M = malloc(sizeof(double) * (size_t)Pp * P * xsize * nmu);
    #pragma omp parallel for collapse(3)
    for (int p = 0; p < Pp; p++)
        for (int q = 0; q < P; q++)
            for (int xi = 0; xi < xsize; xi++) {
                double *vec = malloc(sizeof(double) * (size_t)L);
                for (int l = 0; l < L; l++)
                    vec[l] = (ttw[l] * qt[((long)xi * Pp + p) * (lmax + 1) + lmin + l]) * basis[(long)l * P + q];
                for (int k = 0; k < nmu; k++) {
                    double sum = 0;
                    const double *row = pl + (long)k * (lmax + 1);
                    for (int l = 0; l < L; l++) sum += row[l + lmin] * vec[l];
                    M[(((long)p * P + q) * xsize + xi) * nmu + k] = sum;
                }
                free(vec);
            }
    /* gamma_2d_pt_TTT (:512-555), calculate_gamma_2d (:773-842) */
    #pragma omp parallel for collapse(2) schedule(dynamic, 4)
    for (int m = 0; m < N; m++)
        for (int n = 0; n < Nprim; n++) {
            const int *pp = prim + 3 * n, *qq = triples + 3 * m;
            double *y = malloc(sizeof(double) * (size_t)xsize);
            for (int xi = 0; xi < xsize; xi++) {
#define MT(a, b) (M + (((long)pp[a] * P + qq[b]) * xsize + xi) * nmu)
                const double *m11 = MT(0, 0), *m12 = MT(0, 1), *m13 = MT(0, 2);
                const double *m21 = MT(1, 0), *m22 = MT(1, 1), *m23 = MT(1, 2);
                const double *m31 = MT(2, 0), *m32 = MT(2, 1), *m33 = MT(2, 2);
#undef MT
                double result = 0.0;
                for (int j = 0; j < nmu; j++) {
                    double s1 = m11[j] * m22[j] * m33[j], s2 = m11[j] * m23[j] * m32[j];
                    double s3 = m12[j] * m21[j] * m33[j], s4 = m12[j] * m23[j] * m31[j];
                    double s5 = m13[j] * m21[j] * m32[j], s6 = m13[j] * m22[j] * m31[j];
                    result += w[j] * (s1 + s2 + s3 + s4 + s5 + s6);
                }
                y[xi] = xvec[xi] * xvec[xi] * result;
                if (xi < 10 && fabs(y[xi]) > 1e-18) y[xi] = 0;
            }
            out[(long)m * Nprim + n] = orc_integrate_cubic_spline(xvec, y, xsize) * dphi * dphi / (8.0 * ORC_PI);
            free(y);
        }
    free(ttw); free(pl); free(M);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Polarised late x primordial transfer Gamma: results[1..3] of             */
/* calculate_gamma_2d with do_polarisation (calculate_gamma.c).             */
/*   TTweight_l = (2l+1)^{5/6} b_T / sqrt(s_TT),  s_TT = b_T^2 C_TT + N_TT    */
/*   EEweight_l = (2l+1)^{5/6} b_E / sqrt(s_TT (s_TT s_EE - s_TE^2))         */
/*     s_TE = b_T b_E C_TE + N_TE, s_EE = b_E^2 C_EE + N_EE      (:142-157)   */
/*   q~_E'[x][p][l] = EEweight (s_TT q~_E - (sqrt(fE/fT) b_TE^2 C_TE + N_TE) */
/*                    q~_T)                                      (:170-181)   */
/*   M_T = sum_l P_l TTweight q~_T basis_T, M_E = sum_l P_l q~_E' basis_E    */
/*   TTE/TEE/EEE points: perm3 of [M_{type(b)}[p_a][q_b]] with the late      */
/*   legs' types (T,T,E), (T,E,E), (E,E,E)                  (:558-687)       */
/* then the same x^2, zero rule, spline and dphi^2/(8 pi) as TTT.           */
/* Spectra arrays cover l = 0..max(lmax, lmaxE); lmaxE <= lmax.             */
/* ------------------------------------------------------------------------ */
int orc_gamma_transfer_pol(int lmin, int lmax, int P, const double *basisT, int lminE, int lmaxE, int PE,
                           const double *basisE, int N, const int *tte, const int *tee, const int *eee,
                           const double *cl_tt, const double *cl_te, const double *cl_ee, const double *b_tt,
                           const double *b_te, const double *b_ee, const double *n_tt, const double *n_te,
                           const double *n_ee, double fsky_t, double fsky_e, int nmu, const double *mu,
                           const double *w, int xsize, const double *xvec, int Pp, const double *qtT,
                           const double *qtE, int Nprim, const int *prim, double dphi, double *out /*[3][N][Nprim]*/)
{
    const int L = lmax - lmin + 1, LE = lmaxE - lminE + 1, lstride = lmax + 1;
    double *ttw = malloc(sizeof(double) * (size_t)L), *eew = malloc(sizeof(double) * (size_t)LE);
    for (int i = 0; i < L; i++) {
        int l = lmin + i;
        double s2 = b_tt[l] * b_tt[l] * cl_tt[l] + n_tt[l];
        ttw[i] = (l > 1) ? pow(2e0 * l + 1e0, 5e0 / 6e0) * (b_tt[l] / sqrt(s2)) : 0e0;
    }
    for (int i = 0; i < LE; i++) {
        int l = lminE + i;
        double s2 = b_tt[l] * b_tt[l] * cl_tt[l] + n_tt[l];
        double s3 = b_tt[l] * b_ee[l] * cl_te[l] + n_te[l];
        double s4 = b_ee[l] * b_ee[l] * cl_ee[l] + n_ee[l];
        eew[i] = (l > 1) ? pow(2e0 * l + 1e0, 5e0 / 6e0) * (b_ee[l] / sqrt(s2 * (s2 * s4 - s3 * s3))) : 0e0;
    }
    double *pl = malloc(sizeof(double) * (size_t)nmu * lstride);
    #pragma omp parallel for
    for (int k = 0; k < nmu; k++) {
        double x = mu[k], pm2 = 1.0, pm1 = x;
        double *row = pl + (long)k * lstride;
        for (int l = 0; l <= lmax; l++) {
            double p;
            if (l == 0) p = 1.0;
            else if (l == 1) p = x;
            else {
                double pr = (x * (2 * l - 1) * pm1 - (l - 1) * pm2) / l;
                pm2 = pm1; pm1 = pr;
                p = (l == 2) ? 0.5 * (3.0 * x * x - 1.0) : (x == 1.0 ? 1.0 : (x == -1.0 ? ((l & 1) ? -1.0 : 1.0) : pr));
            }
            row[l] = p;
        }
    }
    double *MT = malloc(sizeof(double) * (size_t)Pp * P * xsize * nmu);
    double *ME = malloc(sizeof(double) * (size_t)Pp * PE * xsize * nmu);
    #pragma omp parallel for collapse(3)
    for (int p = 0; p < Pp; p++)
        for (int xi = 0; xi < xsize; xi++)
            for (int q = 0; q < (P > PE ? P : PE); q++) {
                double *vec = malloc(sizeof(double) * (size_t)(L > LE ? L : LE));
                if (q < P) {
                    for (int l = 0; l < L; l++)
                        vec[l] = (ttw[l] * qtT[((long)xi * Pp + p) * lstride + lmin + l]) * basisT[(long)l * P + q];
                    for (int k = 0; k < nmu; k++) {
                        double sum = 0;
                        for (int l = 0; l < L; l++) sum += pl[(long)k * lstride + l + lmin] * vec[l];
                        MT[(((long)p * P + q) * xsize + xi) * nmu + k] = sum;
                    }
                }
                if (q < PE) {
                    for (int i = 0; i < LE; i++) {
                        int l = lminE + i;
                        double s1 = b_tt[l] * b_tt[l] * cl_tt[l] + n_tt[l];
                        double s2 = sqrt(fsky_e / fsky_t) * b_te[l] * b_te[l] * cl_te[l] + n_te[l];
                        double qe = eew[i] * (s1 * qtE[((long)xi * Pp + p) * lstride + l] - s2 * qtT[((long)xi * Pp + p) * lstride + l]);
                        vec[i] = qe * basisE[(long)i * PE + q];
                    }
                    for (int k = 0; k < nmu; k++) {
                        double sum = 0;
                        for (int i = 0; i < LE; i++) sum += pl[(long)k * lstride + i + lminE] * vec[i];
                        ME[(((long)p * PE + q) * xsize + xi) * nmu + k] = sum;
                    }
                }
                free(vec);
            }
    const int *lists[3] = {tte, tee, eee};
    const int nT[3] = {2, 1, 0};
    #pragma omp parallel for collapse(3) schedule(dynamic, 4)
    for (int f = 0; f < 3; f++)
        for (int m = 0; m < N; m++)
            for (int n = 0; n < Nprim; n++) {
                const int *pp = prim + 3 * n, *qq = lists[f] + 3 * m;
                double *y = malloc(sizeof(double) * (size_t)xsize);
                for (int xi = 0; xi < xsize; xi++) {
                    const double *c[3][3];
                    for (int a = 0; a < 3; a++)
                        for (int b = 0; b < 3; b++)
                            c[a][b] = (b < nT[f]) ? MT + (((long)pp[a] * P + qq[b]) * xsize + xi) * nmu
                                                  : ME + (((long)pp[a] * PE + qq[b]) * xsize + xi) * nmu;
                    double result = 0.0;
                    for (int j = 0; j < nmu; j++) {
                        double s1 = c[0][0][j] * c[1][1][j] * c[2][2][j], s2 = c[0][0][j] * c[1][2][j] * c[2][1][j];
                        double s3 = c[0][1][j] * c[1][0][j] * c[2][2][j], s4 = c[0][1][j] * c[1][2][j] * c[2][0][j];
                        double s5 = c[0][2][j] * c[1][0][j] * c[2][1][j], s6 = c[0][2][j] * c[1][1][j] * c[2][0][j];
                        result += w[j] * (s1 + s2 + s3 + s4 + s5 + s6);
                    }
                    y[xi] = xvec[xi] * xvec[xi] * result;
                    if (xi < 10 && fabs(y[xi]) > 1e-18) y[xi] = 0;
                }
                out[((long)f * N + m) * Nprim + n] = orc_integrate_cubic_spline(xvec, y, xsize) * dphi * dphi / (8.0 * ORC_PI);
                free(y);
            }
    free(ttw); free(eew); free(pl); free(MT); free(ME);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Primordial k-space side: the grid tetrapyd of get_ijk_next_prim           */
/* (tetrapyd_tools.c:485-517, start check_ijk_min_prim :519-550), the cell   */
/* weights of calculate_weight (calculate_volume.c:12-133) and the Gram      */
/* matrix / projection sums of calculate_ortho (orthogonalisation.c:14-86)   */
/* and calculate_eigen / integrate_template2 (calculate_eigen.c:13-144).     */
/* ------------------------------------------------------------------------ */
static double cell1(double a, double b, double c, double d, double e, double f, double g, double h)
{ (void)0; return (11 * (a + b + c + e) + 17 * (d + g + f) + 25 * h) / 240.0; }
static double cell2(double a, double b, double c, double d, double e, double f, double g, double h)
{ return (47 * a + 19 * (b + c + e) + 5 * (d + f + g) + h) / 720.0; }
static double cell3(double a, double b, double c, double d, double e, double f, double g, double h)
{ return (40 * (b + c) + 35 * (a + d) + 26 * (f + g) + 19 * (e + h)) / 360.0; }
static double cell4(double a, double b, double c, double d, double e, double f, double g, double h)
{ return (89 * a + 85 * (b + c + e) + 71 * (d + f + g) + 43 * h) / 720.0; }

double orc_prim_weight(int min, int max, int i, int j, int k)
{
    int grid[3][3][3], sum = 0;
    for (int l = 0; l < 3; l++)
        for (int m = 0; m < 3; m++)
            for (int n = 0; n < 3; n++) {
                const int i0 = i + l - 1, j0 = j + m - 1, k0 = k + n - 1;
                if (i0 < min || i0 > max || j0 < min || j0 > max || k0 < min || k0 > max) grid[l][m][n] = -8;
                else if (i0 > j0 + k0 || j0 > i0 + k0 || k0 > i0 + j0) grid[l][m][n] = 0;
                else { grid[l][m][n] = 1; sum++; }
            }
    double weight = 0.0;
    if (sum == 27) {
        weight = 1.0;
    } else {
        double pt[3][3][3] = {{{0}}};
        pt[1][1][1] = 1.0;
        for (int s1 = 0; s1 < 2; s1++)
            for (int s2 = 0; s2 < 2; s2++)
                for (int s3 = 0; s3 < 2; s3++) {
                    int su = 0;
                    for (int l = 0; l < 2; l++)
                        for (int m = 0; m < 2; m++)
                            for (int n = 0; n < 2; n++) su += grid[l + s1][m + s2][n + s3];
                    const double a = pt[s1][s2][s3], b = pt[s1 + 1][s2][s3], c = pt[s1][s2 + 1][s3],
                                 d = pt[s1 + 1][s2 + 1][s3], e = pt[s1][s2][s3 + 1], f = pt[s1 + 1][s2][s3 + 1],
                                 g = pt[s1][s2 + 1][s3 + 1], h = pt[s1 + 1][s2 + 1][s3 + 1];
                    if (su == 4) {
                        if (grid[1 + s1][0 + s2][1 + s3] == 1) weight += cell2(f, e, h, g, b, a, d, c);
                        if (grid[1 + s1][1 + s2][0 + s3] == 1) weight += cell2(d, c, b, a, h, g, f, e);
                        if (grid[0 + s1][1 + s2][1 + s3] == 1) weight += cell2(g, h, e, f, c, d, a, b);
                    } else if (su == 5) {
                        weight += cell1(a, b, c, d, e, f, g, h);
                    } else if (su == 6) {
                        if (grid[0 + s1][0 + s2][1 + s3] == 1) weight += cell3(g, h, e, f, c, d, a, b);
                        if (grid[1 + s1][0 + s2][0 + s3] == 1) weight += cell3(f, h, b, d, e, g, a, c);
                        if (grid[0 + s1][1 + s2][0 + s3] == 1) weight += cell3(d, h, c, g, b, f, a, e);
                    } else if (su == 7) {
                        if (grid[0 + s1][1 + s2][0 + s3] == 0) weight += cell4(f, e, h, g, b, a, d, c);
                        if (grid[0 + s1][0 + s2][1 + s3] == 0) weight += cell4(d, c, b, a, h, g, f, e);
                        if (grid[1 + s1][0 + s2][0 + s3] == 0) weight += cell4(g, h, e, f, c, d, a, b);
                    } else if (su == 8) {
                        weight += 1.0 / 8.0;
                    }
                }
    }
    if (i != k) weight *= (i == j || j == k) ? 3.0 : 6.0;
    return weight;
}

/* Walk of get_ijk_next_prim from the start of check_ijk_min_prim: writes up
 * to cap points (i,j,k) and returns how many decompose_tetrapyd_prim counts
 * (all the points with i < max, then the end point (max,max,max)). */
long orc_prim_walk(int min, int max, long cap, int *pts)
{
    int i = min, j = min, k = min;
    if (i + j + 2 < k) k = i + j + 2;
    long n = 0;
    for (;;) {
        if (n < cap) { pts[3 * n] = i; pts[3 * n + 1] = j; pts[3 * n + 2] = k; }
        n++;
        if (j == max) { i++; j = i; k = j; }
        else if (k == max || k >= i + j + 2) { j++; k = j; }
        else k++;
        if (i >= max) {
            if (n < cap) { pts[3 * n] = max; pts[3 * n + 1] = max; pts[3 * n + 2] = max; }
            return n + 1;
        }
    }
}

static double prim_pijk(const double *basis, int P, const int *tr, int i, int j, int k)
{
#define BP(l, p) basis[(long)(l) * P + (p)]
    const int p1 = tr[0], p2 = tr[1], p3 = tr[2];
    double b1 = BP(i, p1) * BP(j, p2) * BP(k, p3), b2 = BP(i, p2) * BP(j, p3) * BP(k, p1);
    double b3 = BP(i, p3) * BP(j, p1) * BP(k, p2), b4 = BP(i, p3) * BP(j, p2) * BP(k, p1);
    double b5 = BP(i, p2) * BP(j, p1) * BP(k, p3), b6 = BP(i, p1) * BP(j, p3) * BP(k, p2);
#undef BP
    return (b1 + b2 + b3 + b4 + b5 + b6) / 6.0;
}

static double prim_point_weight(int min, int max, double kmax, int i, int j, int k)
{
    const double factor = kmax * (1e0 / (double)max), cube = factor * factor * factor;
    double x = orc_prim_weight(min, max, i, j, k) * cube;
    double ksum = factor * i + factor * j + factor * k;
    if (ksum > 1e-10) ksum = 1e0 / ksum;
    return x * ksum;
}

int orc_prim_ortho(int min, int max, double kmax, int P, const double *basis, int N, const int *prim, double *out)
{
    long npts = orc_prim_walk(min, max, 0, NULL);
    int *pts = malloc(sizeof(int) * 3 * (size_t)npts);
    orc_prim_walk(min, max, npts, pts);
    const long vsize = (long)N * (N + 1) / 2;
    for (long v = 0; v < vsize; v++) out[v] = 0.0;
    double *b = malloc(sizeof(double) * (size_t)N);
    for (long n = 0; n < npts; n++) {
        const int i = pts[3 * n], j = pts[3 * n + 1], k = pts[3 * n + 2];
        const double x = prim_point_weight(min, max, kmax, i, j, k);
        for (int r = 0; r < N; r++) b[r] = prim_pijk(basis, P, prim + 3 * r, i, j, k);
        long m = 0;
        for (int r = 0; r < N; r++)
            for (int s = r; s < N; s++) out[m++] += x * b[r] * b[s];
    }
    free(b);
    free(pts);
    return 0;
}

int orc_prim_eigen(int min, int max, double kmax, int P, const double *basis, int N, const int *prim, int kind,
                   int nterms, const double *tab, double c1, double c2, double c3, double sigma, double *alpha,
                   double *norm2)
{
    orc_shape sh = {kind, nterms, max, tab, c1, c2, c3, sigma};
    long npts = orc_prim_walk(min, max, 0, NULL);
    int *pts = malloc(sizeof(int) * 3 * (size_t)npts);
    orc_prim_walk(min, max, npts, pts);
    for (int r = 0; r < N; r++) alpha[r] = 0.0;
    double y = 0.0;
    for (long n = 0; n < npts; n++) {
        const int i = pts[3 * n], j = pts[3 * n + 1], k = pts[3 * n + 2];
        const double x = prim_point_weight(min, max, kmax, i, j, k);
        const double s = orc_shape_eval(&sh, i, j, k);
        for (int r = 0; r < N; r++) alpha[r] += (x * s) * prim_pijk(basis, P, prim + 3 * r, i, j, k);
        y += x * (s * s);
    }
    *norm2 = y;
    free(pts);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* 3D transfer Gamma (calculate_gamma_3d.c): calculate_gamma_TTT_3D_nested    */
/* (:274-440) over the tetrapyd of gamma_3d_host (gamma_mpi.c:30-152) with    */
/* the point set of decompose_gamma_TTT_3D_mpi (:92-211):                     */
/*   Gamma[m][n] = 6 dphi^2 sum_pts z plijk_m(i,j,k) s_n(i,j,k),              */
/*   z = permsix h~^2 prod (2l+1)^{-1/3} (lweight3D, init_gamma_3Dint :23-44),*/
/*   s_n = trapezium over x of x^2 (1/6) sum_perms q3(i,a1) q3(j,a2) q3(k,a3) */
/*   (calculate_sijk_TTT :813-860, integrate :783-811), the first 10 samples  */
/*   dropped where |y| > 1e-18; q3(l,a,x) = (2l+1)^{1/6}/sqrt(cl[l]) q~_a(l,x)*/
/*   for l > 1 (init_gamma_3Dint :46-60).  Points i = 2..lmax, j = i..lmax,   */
/*   k = j + (i % 2) .. min(i + j, lmax) step 2.  out[N][Nprim].             */
/* ------------------------------------------------------------------------ */
int orc_gamma_3d(int lmin, int lmax, int P, const double *basis, int N, const int *triples, const double *cl, int xsize,
                 const double *xvec, int Pp, const double *qt, int Nprim, const int *prim, double dphi, double *out)
{
    const int L1 = lmax + 1;
    double *lw = malloc(sizeof(double) * L1), *wq = malloc(sizeof(double) * L1);
    for (int l = 0; l <= lmax; l++) {
        lw[l] = l > 1 ? 1e0 / pow(2e0 * l + 1e0, 1e0 / 3e0) : 0e0;
        wq[l] = l > 1 ? pow(2e0 * l + 1e0, 1e0 / 6e0) * (1e0 / sqrt(cl[l])) : 0e0;
    }
    const int nth = omp_get_max_threads();
    double *acc = calloc((size_t)nth * N * Nprim, sizeof(double));
    #pragma omp parallel
    {
        const int t = omp_get_thread_num();
        double *g = acc + (size_t)t * N * Nprim;
        double *y = malloc(sizeof(double) * xsize), *s = malloc(sizeof(double) * Nprim), *Q = malloc(sizeof(double) * N);
        #pragma omp for schedule(dynamic, 1)
        for (int i = 2; i <= lmax; i++)
            for (int j = i; j <= lmax; j++)
                for (int k = j + (i % 2); k <= (i + j < lmax ? i + j : lmax); k += 2) {
                    const double z = orc_permsix(i, j, k) * orc_geometric(i, j, k) * lw[i] * lw[j] * lw[k];
                    for (int n = 0; n < Nprim; n++) {
                        const int a1 = prim[3 * n], a2 = prim[3 * n + 1], a3 = prim[3 * n + 2];
                        for (int x = 0; x < xsize; x++) {
                            const double *qx = qt + (size_t)x * Pp * L1;
                            const double p1 = wq[i] * qx[(size_t)a1 * L1 + i], p2 = wq[i] * qx[(size_t)a2 * L1 + i],
                                         p3 = wq[i] * qx[(size_t)a3 * L1 + i];
                            const double p4 = wq[j] * qx[(size_t)a1 * L1 + j], p5 = wq[j] * qx[(size_t)a2 * L1 + j],
                                         p6 = wq[j] * qx[(size_t)a3 * L1 + j];
                            const double p7 = wq[k] * qx[(size_t)a1 * L1 + k], p8 = wq[k] * qx[(size_t)a2 * L1 + k],
                                         p9 = wq[k] * qx[(size_t)a3 * L1 + k];
                            const double sum = p1 * p5 * p9 + p2 * p6 * p7 + p3 * p4 * p8 + p3 * p5 * p7 + p2 * p4 * p9 +
                                               p1 * p6 * p8;
                            double v = xvec[x] * xvec[x] * sum * (1e0 / 6e0);
                            if (x < 10 && fabs(v) > 1e-18) v = 0e0;
                            y[x] = v;
                        }
                        double r = 0e0;
                        for (int x = 0; x < xsize - 1; x++) r += (xvec[x + 1] - xvec[x]) * (y[x] + y[x + 1]) * 0.5;
                        s[n] = r;
                    }
                    for (int m = 0; m < N; m++) Q[m] = plijk(basis, P, triples + 3 * m, lmin, lmax, i, j, k) * z;
                    for (int m = 0; m < N; m++)
                        for (int n = 0; n < Nprim; n++) g[(size_t)m * Nprim + n] += Q[m] * s[n];
                }
        free(y); free(s); free(Q);
    }
    const double f = 6e0 * dphi * dphi;
    for (size_t e = 0; e < (size_t)N * Nprim; e++) {
        double v = 0e0;
        for (int t = 0; t < nth; t++) v += acc[(size_t)t * N * Nprim + e];
        out[e] = v * f;
    }
    free(acc); free(lw); free(wq);
    return 0;
}
