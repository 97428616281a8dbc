/*
 * tv_fb_oracle.c -- CPU restatement of the reference's HSMM forward-backward.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the GPU forward-backward
 * (tensor-viterbi_gb300/csrc/tv_fb.cuh).  No product code path links, loads
 * or calls it.
 *
 * It restates, in plain C with IEEE double arithmetic and the same loops and
 * association, hsmmlearn's FBImpl (hsmmlearn/hsmmlearn/_hsmm/src/FBImpl.cpp,
 * with CalcStoreD of dCalc.cpp and the argument layout of InitData.cpp), the
 * E step that hsmmlearn's HSMMModel.fit (hsmmlearn/hsmmlearn/hsmm.py:181-305)
 * calls once per EM iteration.  Censoring 0 (none) and 1 (right censoring,
 * the fit's default) are stated; the left-censoring variant (2) is not.
 *
 * Layouts (InitData.cpp:154-173): d (J, M) duration pmf rows, entry u-1 the
 * probability of duration u; p (J, J) transition matrix [from][to]; pi (J);
 * pdf (J, tau) observation likelihoods.  Outputs (J, tau): F, L, G (column 0
 * unset), L1 (column tau-1 unset), Norm; N (tau); eta (J, M).
 * Returns 0, or 1 where the reference throws var_nonpositive_exception
 * (a normaliser N[t] or a forward variable F[j][t] not positive).
 */
#include <stdlib.h>
#include <string.h>

#define AT(a, j, t) a[(size_t)(j) * tau + (t)]

static int imin(int a, int b) { return a < b ? a : b; }

int tvo_fb(int censoring, int tau, int J, int M, const double* dpara, const double* p, const double* pi,
           const double* pdf, double* F, double* L, double* G, double* L1, double* Nn, double* Norm,
           double* eta) {
    if (tau < 1 || J < 1 || M < 1 || (censoring != 0 && censoring != 1)) return -1;
    const int right = censoring == 1;
    const int dl = (M + 1 > tau ? M + 1 : tau + 1);
    double* d = (double*)calloc((size_t)J * (M + 1), sizeof(double));   /* d[j][u], u = 1..M */
    double* D = (double*)calloc((size_t)J * dl, sizeof(double));        /* D[j][u], u = 1..max(M, tau) */
    double* S = (double*)calloc((size_t)J * tau, sizeof(double));       /* StateIn */
    double* H = (double*)calloc((size_t)J * tau * (M + 1), sizeof(double));
    int rc = 0;
    if (!d || !D || !S || !H) { rc = -2; goto out; }
#define Dd(j, u) d[(size_t)(j) * (M + 1) + (u)]
#define DD(j, u) D[(size_t)(j) * dl + (u)]
#define HH(j, t, u) H[((size_t)(j) * tau + (t)) * (M + 1) + (u)]
    for (int j = 0; j < J; ++j)
        for (int u = 0; u < M; ++u) Dd(j, u + 1) = dpara[(size_t)j * M + u];
    /* CalcStoreD (dCalc.cpp:5-30): survival D[j][u] = sum_{v >= u} d[j][v] */
    for (int j = 0; j < J; ++j) {
        for (int u = 1; u <= M; ++u) {
            double x = 0;
            for (int v = u; v < M + 1; ++v) x += Dd(j, v);
            DD(j, u) = x;
        }
        for (int u = M + 1; u <= tau; ++u) DD(j, u) = 0;
    }

    /* forward recursion (FBImpl.cpp:62-140) */
    for (int t = 0; t <= tau - 1; ++t) {
        Nn[t] = 0;
        for (int j = 0; j <= J - 1; ++j) {
            if (t == 0)
                AT(Norm, j, 0) = AT(pdf, j, 0) * pi[j];
            else
                AT(Norm, j, t) = AT(pdf, j, t) * (AT(S, j, t) - AT(F, j, t - 1) + AT(Norm, j, t - 1));
            Nn[t] += AT(Norm, j, t);
        }
        if (Nn[t] <= 0) { rc = 1; goto out; }
        for (int j = 0; j <= J - 1; ++j) AT(Norm, j, t) /= Nn[t];
        for (int j = 0; j <= J - 1; ++j) {
            AT(F, j, t) = 0;
            double Observ = 1;
            if (t < tau - 1) {
                for (int u = 1; u <= imin(t + 1, M); ++u) {
                    Observ *= AT(pdf, j, t - u + 1) / Nn[t - u + 1];
                    if (u < t + 1)
                        AT(F, j, t) += Observ * Dd(j, u) * AT(S, j, t - u + 1);
                    else
                        AT(F, j, t) += Observ * Dd(j, t + 1) * pi[j];
                }
            } else {
                for (int u = 1; u <= imin(tau, M); ++u) {
                    Observ *= AT(pdf, j, tau - u) / Nn[tau - u];
                    if (u < tau)
                        AT(F, j, tau - 1) += Observ * DD(j, u) * AT(S, j, tau - u);
                    else
                        AT(F, j, tau - 1) += Observ * DD(j, tau) * pi[j];
                }
            }
            if (AT(F, j, t) <= 0) { rc = 1; goto out; }
        }
        if (t < tau - 1)
            for (int j = 0; j <= J - 1; ++j) {
                AT(S, j, t + 1) = 0;
                for (int i = 0; i <= J - 1; ++i) AT(S, j, t + 1) += p[(size_t)i * J + j] * AT(F, i, t);
            }
    }

    /* backward recursion (FBImpl.cpp:142-178) */
    for (int j = 0; j <= J - 1; ++j) AT(L, j, tau - 1) = AT(F, j, tau - 1);
    for (int t = tau - 2; t >= 0; --t) {
        for (int j = 0; j <= J - 1; ++j) {
            AT(G, j, t + 1) = 0;
            double Observ = 1;
            for (int u = 1; u <= imin(tau - 1 - t, M); ++u) {
                Observ *= AT(pdf, j, t + u) / Nn[t + u];
                if (u < tau - 1 - t)
                    HH(j, t + 1, u) = AT(L1, j, t + u) * Observ * Dd(j, u) / AT(F, j, t + u);
                else
                    HH(j, t + 1, u) = Observ * DD(j, tau - 1 - t);
                AT(G, j, t + 1) += HH(j, t + 1, u);
            }
        }
        for (int j = 0; j <= J - 1; ++j) {
            AT(L1, j, t) = 0;
            for (int k = 0; k <= J - 1; ++k) AT(L1, j, t) += AT(G, k, t + 1) * p[(size_t)j * J + k];
            AT(L1, j, t) *= AT(F, j, t);
            AT(L, j, t) = AT(L1, j, t) + AT(L, j, t + 1) - AT(G, j, t + 1) * AT(S, j, t + 1);
        }
    }

    /* eta without left censoring (FBImpl.cpp:231-270) */
    for (int j = 0; j <= J - 1; ++j) {
        for (int u = 1; u <= M; ++u) {
            double w = 0, s = 1, r;
            for (int t = tau - 2 - (right ? 0 : 1) * u; t >= 0; --t) {
                r = 0;
                for (int i = 0; i <= J - 1; ++i)
                    if (i != j) r += p[(size_t)i * J + j] * AT(F, i, t);
                if (u <= tau - 2 - t) {
                    r *= HH(j, t + 1, u);
                } else {
                    s *= AT(pdf, j, t + 1) / Nn[t + 1];
                    r *= s * Dd(j, u);
                }
                w += r;
            }
            if (right || u <= tau - 1) {
                r = Dd(j, u) * pi[j];
                if (u <= tau - 1) {
                    for (int v = 1; v <= u; ++v) r *= AT(pdf, j, u - v) / Nn[u - v];
                    r *= AT(L1, j, u - 1) / AT(F, j, u - 1);
                } else {
                    for (int v = 1; v <= tau; ++v) r *= AT(pdf, j, tau - v) / Nn[tau - v];
                }
                w += r;
            }
            eta[(size_t)j * M + (u - 1)] = w;
        }
    }
out:
    free(d);
    free(D);
    free(S);
    free(H);
    return rc;
}
