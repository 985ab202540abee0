/*
 * pf2_oracle_solvers.c - solver options of the engine beyond the reference, restated on
 * the CPU (TEST INFRASTRUCTURE ONLY: the checker of the tests and the CPU leg of the
 * benchmark, never part of the product).
 *
 * The reference solves the pressure with CG and ILU(0)/IC(0) in the natural row order
 * (src/linear_algebra/linear_solver.cu:301-376, preconditioners.cu:48-213) and the
 * velocity prediction with unrestarted GMRES and modified Gram-Schmidt
 * (linear_solver.cu:378-521).  The engine adds, as options:
 *  - ILU(0)/IC(0) on a multicolour permutation B = P A P^T (greedy colouring in row
 *    order, the thin tail of high colours moved down by Kempe-chain swaps);
 *  - a relative stopping test ||r|| <= tol ||b|| beside the reference's absolute one;
 *  - right-preconditioned BiCGStab (van der Vorst, SIAM J. Sci. Stat. Comput. 13 (1992),
 *    Alg. 3.1 with a right preconditioner) for the nonsymmetric prediction systems;
 *  - GMRES with classical Gram-Schmidt applied twice (Daniel, Gragg, Kaufman and
 *    Stewart, Math. Comp. 30 (1976): a second pass only when the first left less than
 *    0.7 of the vector's norm).
 * These are the published algorithms, written here for the CPU so that the oracle can
 * run the step with the same solver choices as the engine.
 *
 * Threads: rows of a colour are independent, so the multicolour sweeps, the SpMV and
 * the vector updates run under OpenMP without changing any bit.  Dot products are
 * summed over fixed 4,096-row chunks in chunk order, so their bits do not depend on
 * the thread count either.
 */
#include "pf2_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define PAR_MIN 32768
#define CHUNK 4096

static double pdot(int n, const double* a, const double* b)
{
    const int nch = (n + CHUNK - 1) / CHUNK;
    double stack[256];
    double* part = nch <= 256 ? stack : (double*)malloc(sizeof(double) * nch);
#pragma omp parallel for schedule(static) if (n > PAR_MIN)
    for (int c = 0; c < nch; ++c) {
        const int i1 = (c + 1) * CHUNK < n ? (c + 1) * CHUNK : n;
        double s = 0.0;
        for (int i = c * CHUNK; i < i1; ++i) s += a[i] * b[i];
        part[c] = s;
    }
    double s = 0.0;
    for (int c = 0; c < nch; ++c) s += part[c];
    if (part != stack) free(part);
    return s;
}

/* ------------------------------------------------------------------ ordering */

/* Kempe-chain trimming of a greedy colouring (nc colours): every node of the thin tail
 * of high colours (colours K.. with fewer than max(1, n / 500) nodes together) is moved
 * below K.  For a tail node v, colours a < K are tried in turn: a is taken directly
 * when no neighbour has it; otherwise, for each b < K, b != a, the (a, b)-Kempe chain
 * grown from v's a-coloured neighbours (breadth first, in CSR order) is swapped when it
 * reaches no b-coloured neighbour of v, and v takes a.  Up to four passes over the nodes
 * in index order, stopping when a pass fixes nothing or leaves nothing; 64 n chain
 * visits at most.  Returns the number of colours used. */
static int kempe_trim(int n, const int* rp, const int* col, int* color, int nc)
{
    long long* size = (long long*)calloc(nc, sizeof(long long));
    for (int i = 0; i < n; ++i) size[color[i]]++;
    int K = nc;
    long long tail = 0;
    const long long thin = n / 500 > 1 ? n / 500 : 1;
    while (K > 1 && tail + size[K - 1] < thin) tail += size[--K];
    free(size);
    if (K == nc) return nc;
    int* mark = (int*)malloc(sizeof(int) * n);
    for (int i = 0; i < n; ++i) mark[i] = -1;
    int* queue = (int*)malloc(sizeof(int) * n);
    long long budget = 64LL * n;
    int stamp = 0;
    for (int pass = 0; pass < 4 && budget > 0; ++pass) {
        int left = 0, fixed = 0;
        for (int v = 0; v < n && budget > 0; ++v) {
            if (color[v] < K) continue;
            int done = 0, out_of_budget = 0;
            for (int a = 0; a < K && !done && !out_of_budget; ++a) {
                int has_a = 0;
                for (int k = rp[v]; k < rp[v + 1]; ++k) has_a |= col[k] != v && color[col[k]] == a;
                if (!has_a) { color[v] = a; done = 1; break; }
                for (int b = 0; b < K && !done && !out_of_budget; ++b) {
                    if (b == a) continue;
                    ++stamp;
                    int qn = 0;
                    for (int k = rp[v]; k < rp[v + 1]; ++k)
                        if (col[k] != v && color[col[k]] == a && mark[col[k]] != stamp) {
                            mark[col[k]] = stamp;
                            queue[qn++] = col[k];
                        }
                    int ok = 1;
                    for (int h = 0; h < qn && ok; ++h) {
                        const int x = queue[h];
                        if (--budget < 0) { out_of_budget = 1; break; }
                        for (int k = rp[x]; k < rp[x + 1]; ++k) {
                            const int y = col[k];
                            if (y == x || y == v || mark[y] == stamp) continue;
                            if (color[y] != a && color[y] != b) continue;
                            int nb_of_v = 0;
                            for (int q = rp[v]; q < rp[v + 1]; ++q) nb_of_v |= col[q] == y;
                            if (nb_of_v && color[y] == b) { ok = 0; break; }
                            mark[y] = stamp;
                            queue[qn++] = y;
                        }
                    }
                    if (out_of_budget || !ok) continue;
                    for (int h = 0; h < qn; ++h) color[queue[h]] = color[queue[h]] == a ? b : a;
                    color[v] = a;
                    done = 1;
                }
            }
            if (done) ++fixed;
            else ++left;
        }
        if (left == 0 || fixed == 0) break;
    }
    free(mark);
    free(queue);
    int m = 0;
    for (int i = 0; i < n; ++i) m = color[i] + 1 > m ? color[i] + 1 : m;
    return m;
}

int or_multicolour_order(int n, const int* rp, const int* col, int kempe, int* perm, int* starts)
{
    int* color = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
    char* used = (char*)calloc(n + 1, 1);
    int nc = 0;
    for (int i = 0; i < n; ++i) {
        for (int k = rp[i]; k < rp[i + 1]; ++k)
            if (col[k] < i) used[color[col[k]]] = 1;
        int c = 0;
        while (used[c]) ++c;
        color[i] = c;
        if (c + 1 > nc) nc = c + 1;
        for (int k = rp[i]; k < rp[i + 1]; ++k)
            if (col[k] < i) used[color[col[k]]] = 0;
    }
    free(used);
    if (kempe) nc = kempe_trim(n, rp, col, color, nc);
    int* cnt = (int*)calloc(nc + 1, sizeof(int));
    for (int i = 0; i < n; ++i) cnt[color[i] + 1]++;
    for (int c = 0; c < nc; ++c) cnt[c + 1] += cnt[c];
    if (starts) memcpy(starts, cnt, sizeof(int) * (nc + 1));
    for (int i = 0; i < n; ++i) perm[cnt[color[i]]++] = i;
    free(cnt);
    free(color);
    return nc;
}

/* B = P A P^T: row r of B is row perm[r] of A, columns renumbered and sorted. */
typedef struct {
    int n, ngroups;
    int *perm, *iperm, *starts;
    int *rp, *col;
    double* val;
} permuted;

static int cmp_pair(const void* a, const void* b)
{
    const int x = ((const int*)a)[0], y = ((const int*)b)[0];
    return (x > y) - (x < y);
}

static void permute_init(permuted* B, int n, const int* rp, const int* col, const double* val, int multicolour)
{
    B->n = n;
    B->perm = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
    B->iperm = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
    B->starts = (int*)malloc(sizeof(int) * (n + 2));
    if (multicolour) {
        B->ngroups = or_multicolour_order(n, rp, col, 1, B->perm, B->starts);
    } else {
        for (int i = 0; i < n; ++i) B->perm[i] = i;
        B->ngroups = n; /* one row per group: the sequential sweep */
        for (int i = 0; i <= n; ++i) B->starts[i] = i;
    }
    for (int r = 0; r < n; ++r) B->iperm[B->perm[r]] = r;
    const int nnz = rp[n];
    B->rp = (int*)malloc(sizeof(int) * (n + 1));
    B->col = (int*)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
    B->val = (double*)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
    B->rp[0] = 0;
    for (int r = 0; r < n; ++r) B->rp[r + 1] = B->rp[r] + (rp[B->perm[r] + 1] - rp[B->perm[r]]);
#pragma omp parallel if (n > PAR_MIN)
    {
        int cap = 64;
        int* pair = (int*)malloc(sizeof(int) * 2 * cap);
#pragma omp for schedule(static)
        for (int r = 0; r < n; ++r) {
            const int o = B->perm[r], len = rp[o + 1] - rp[o];
            if (len > cap) {
                cap = len;
                pair = (int*)realloc(pair, sizeof(int) * 2 * cap);
            }
            for (int k = 0; k < len; ++k) {
                pair[2 * k] = B->iperm[col[rp[o] + k]];
                pair[2 * k + 1] = rp[o] + k;
            }
            qsort(pair, len, 2 * sizeof(int), cmp_pair);
            for (int k = 0; k < len; ++k) {
                B->col[B->rp[r] + k] = pair[2 * k];
                B->val[B->rp[r] + k] = val[pair[2 * k + 1]];
            }
        }
        free(pair);
    }
}

static void permute_free(permuted* B)
{
    free(B->perm); free(B->iperm); free(B->starts); free(B->rp); free(B->col); free(B->val);
}

/* ------------------------------------------------------ preconditioner apply */

typedef struct {
    int kind, n, ngroups;
    const int *rp, *col, *starts;
    double* fact;  /* ILU: L\U; IC: L in the lower part */
    int* tpos;     /* IC: for an upper entry (i, j) of row i, the position of (j, i) in row j */
    int* dpos;
    double* invdiag;
    double* tmp;
} precond;

static void precond_setup(precond* M, int kind, int n, const int* rp, const int* col, const double* val,
                          int ngroups, const int* starts)
{
    memset(M, 0, sizeof(*M));
    M->kind = kind;
    M->n = n;
    M->rp = rp;
    M->col = col;
    M->ngroups = ngroups;
    M->starts = starts;
    M->tmp = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    M->dpos = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
    for (int i = 0; i < n; ++i) M->dpos[i] = or_find_in_row(rp, col, i, i);
    if (kind == OR_PRECOND_JACOBI) {
        M->invdiag = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
        for (int i = 0; i < n; ++i) M->invdiag[i] = M->dpos[i] >= 0 ? 1.0 / val[M->dpos[i]] : 0.0;
    } else if (kind == OR_PRECOND_ILU || kind == OR_PRECOND_IC) {
        const int nnz = rp[n];
        M->fact = (double*)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
        memcpy(M->fact, val, sizeof(double) * nnz);
        if (kind == OR_PRECOND_ILU) or_ilu0(n, rp, col, M->fact);
        else {
            or_ic0(n, rp, col, M->fact);
            M->tpos = (int*)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
            for (int i = 0; i < n; ++i)
                for (int k = rp[i]; k < rp[i + 1]; ++k)
                    M->tpos[k] = col[k] > i ? or_find_in_row(rp, col, col[k], i) : -1;
        }
    }
}

static void precond_release(precond* M)
{
    free(M->fact); free(M->tpos); free(M->dpos); free(M->invdiag); free(M->tmp);
}

/* dst = M^{-1} src.  The triangular sweeps go group by group (forward) and back
 * (backward); the rows of a group do not depend on one another. */
static void precond_apply(const precond* M, const double* src, double* dst)
{
    const int n = M->n;
    const int *rp = M->rp, *col = M->col;
    if (M->kind == OR_PRECOND_NONE) { memmove(dst, src, sizeof(double) * n); return; }
    if (M->kind == OR_PRECOND_JACOBI) {
#pragma omp parallel for schedule(static) if (n > PAR_MIN)
        for (int i = 0; i < n; ++i) dst[i] = src[i] * M->invdiag[i];
        return;
    }
    const int ic = M->kind == OR_PRECOND_IC;
    double* t = M->tmp;
    const double* f = M->fact;
    if (M->ngroups == n) { /* one row per group: the sequential sweeps of the natural order */
        for (int i = 0; i < n; ++i) {
            double s = src[i];
            for (int k = rp[i]; k < M->dpos[i]; ++k) s -= f[k] * t[col[k]];
            t[i] = ic ? s / f[M->dpos[i]] : s;
        }
        for (int i = n - 1; i >= 0; --i) {
            double s = t[i];
            const int d = M->dpos[i];
            if (ic)
                for (int k = d + 1; k < rp[i + 1]; ++k) s -= f[M->tpos[k]] * dst[col[k]];
            else
                for (int k = d + 1; k < rp[i + 1]; ++k) s -= f[k] * dst[col[k]];
            dst[i] = s / f[d];
        }
        return;
    }
    for (int g = 0; g < M->ngroups; ++g) {
        const int r0 = M->starts[g], r1 = M->starts[g + 1];
#pragma omp parallel for schedule(static) if (r1 - r0 > PAR_MIN / 4)
        for (int i = r0; i < r1; ++i) {
            double s = src[i];
            for (int k = rp[i]; k < M->dpos[i]; ++k) s -= f[k] * t[col[k]];
            t[i] = ic ? s / f[M->dpos[i]] : s;
        }
    }
    for (int g = M->ngroups - 1; g >= 0; --g) {
        const int r0 = M->starts[g], r1 = M->starts[g + 1];
#pragma omp parallel for schedule(static) if (r1 - r0 > PAR_MIN / 4)
        for (int i = r0; i < r1; ++i) {
            double s = t[i];
            const int d = M->dpos[i];
            if (ic)
                for (int k = d + 1; k < rp[i + 1]; ++k) s -= f[M->tpos[k]] * dst[col[k]];
            else
                for (int k = d + 1; k < rp[i + 1]; ++k) s -= f[k] * dst[col[k]];
            dst[i] = s / f[d];
        }
    }
}

/* ---------------------------------------------------------------------- CG */

/* PCG as SolverCG::solve (linear_solver.cu:301-376) on B = P A P^T when ordering is
 * multicolour (x and b permuted on the way in and out); x0 is the incoming x.  Stops on
 * r^T z < tol^2 (criterion 0, the reference's) or ||r|| <= tol ||b|| (criterion 1).
 * info->residual: sqrt(r^T z) or ||r|| / ||b||; rel_residual (may be NULL):
 * ||r|| / ||b|| of the recursively updated residual at the end. */
int or_cg(int n, const int* rowptr, const int* col, const double* val, double* x, const double* b, double tol,
          int maxit, int precond_kind, int ordering, int criterion, or_solve_info* info, double* rel_residual)
{
    const int tri = precond_kind == OR_PRECOND_ILU || precond_kind == OR_PRECOND_IC;
    permuted B;
    permute_init(&B, n, rowptr, col, val, tri && ordering == 1);
    precond M;
    precond_setup(&M, precond_kind, n, B.rp, B.col, B.val, B.ngroups, B.starts);
    double* xb = (double*)malloc(sizeof(double) * (n > 0 ? n : 1) * 6);
    double *bb = xb + n, *r = bb + n, *z = r + n, *p = z + n, *q = p + n;
    for (int i = 0; i < n; ++i) {
        xb[i] = x[B.perm[i]];
        bb[i] = b[B.perm[i]];
    }
    or_spmv(n, B.rp, B.col, B.val, xb, q);
#pragma omp parallel for schedule(static) if (n > PAR_MIN)
    for (int i = 0; i < n; ++i) r[i] = bb[i] - q[i];
    precond_apply(&M, r, z);
    memcpy(p, z, sizeof(double) * n);
    const double bnorm = sqrt(pdot(n, bb, bb));
    double gamma = pdot(n, r, z), rr = pdot(n, r, r);
    const double tol2 = tol * tol;
#define CG_DONE(g_, rr_) (criterion == 1 ? sqrt(rr_) <= tol * bnorm : (g_) < tol2)
    int it = 0, conv = CG_DONE(gamma, rr);
    while (!conv && it < maxit) {
        ++it;
        or_spmv(n, B.rp, B.col, B.val, p, q);
        const double alpha = gamma / pdot(n, p, q);
#pragma omp parallel for schedule(static) if (n > PAR_MIN)
        for (int i = 0; i < n; ++i) {
            xb[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        precond_apply(&M, r, z);
        const double gold = gamma;
        gamma = pdot(n, r, z);
        rr = pdot(n, r, r);
        if (CG_DONE(gamma, rr)) { conv = 1; break; }
        const double beta = gamma / gold;
#pragma omp parallel for schedule(static) if (n > PAR_MIN)
        for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
#undef CG_DONE
    for (int i = 0; i < n; ++i) x[B.perm[i]] = xb[i];
    if (info) {
        info->iterations = it;
        info->converged = conv;
        info->residual = criterion == 1 ? sqrt(rr) / (bnorm > 0 ? bnorm : 1.0) : sqrt(gamma);
    }
    if (rel_residual) *rel_residual = sqrt(rr) / (bnorm > 0 ? bnorm : 1.0);
    free(xb);
    precond_release(&M);
    permute_free(&B);
    return conv;
}

/* ---------------------------------------------------------------- BiCGStab */

/* Right-preconditioned BiCGStab (Jacobi or none), x0 the incoming x, rhat = r0.  Stops on
 * ||M^{-1} r|| < tol (criterion 0: the preconditioned residual the reference's GMRES
 * tests, linear_solver.cu:500-505) or ||r|| <= tol ||b|| (criterion 1).  A zero rhat.v
 * ends the solve unconverged; t = A M^{-1} s = 0 takes the half step x += alpha y
 * (omega = 0) and lets the test decide; rhat.r = 0 with r != 0 restarts the shadow
 * residual (rhat = r). */
int or_bicgstab(int n, const int* rowptr, const int* col, const double* val, double* x, const double* b,
                double tol, int maxit, int precond_kind, int criterion, or_solve_info* info)
{
    precond M;
    precond_setup(&M, precond_kind == OR_PRECOND_JACOBI ? OR_PRECOND_JACOBI : OR_PRECOND_NONE, n, rowptr, col,
                  val, 0, NULL);
    const int jac = precond_kind == OR_PRECOND_JACOBI;
    double* w = (double*)malloc(sizeof(double) * (n > 0 ? n : 1) * 8);
    double *r = w, *rhat = r + n, *p = rhat + n, *v = p + n, *y = v + n, *s = y + n, *zz = s + n, *t = zz + n;
    or_spmv(n, rowptr, col, val, x, v);
    double mm = 0.0;
    for (int i = 0; i < n; ++i) {
        r[i] = b[i] - v[i];
        rhat[i] = r[i];
        p[i] = 0.0;
        v[i] = 0.0;
        const double mi = jac ? r[i] * M.invdiag[i] : r[i];
        mm += mi * mi;
    }
    const double bnorm = sqrt(pdot(n, b, b));
    double rho = pdot(n, rhat, r), rr = pdot(n, r, r);
#define BI_DONE(rr_, mm_) (criterion == 1 ? sqrt(rr_) <= tol * bnorm : sqrt(mm_) < tol)
    double rho_old = 1.0, alpha = 1.0, omega = 1.0;
    int it = 0, conv = BI_DONE(rr, mm);
    while (!conv && it < maxit) {
        ++it;
        const double beta = (rho / rho_old) * (alpha / omega);
#pragma omp parallel for schedule(static) if (n > PAR_MIN)
        for (int i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * v[i]);
        precond_apply(&M, p, y);
        or_spmv(n, rowptr, col, val, y, v);
        const double rv = pdot(n, rhat, v);
        if (rv == 0.0) break;
        alpha = rho / rv;
#pragma omp parallel for schedule(static) if (n > PAR_MIN)
        for (int i = 0; i < n; ++i) s[i] = r[i] - alpha * v[i];
        precond_apply(&M, s, zz);
        or_spmv(n, rowptr, col, val, zz, t);
        const double ts = pdot(n, t, s), tt = pdot(n, t, t);
        omega = tt == 0.0 ? 0.0 : ts / tt;
#pragma omp parallel for schedule(static) if (n > PAR_MIN)
        for (int i = 0; i < n; ++i) {
            x[i] += alpha * y[i] + omega * zz[i];
            r[i] = s[i] - omega * t[i];
        }
        precond_apply(&M, r, s); /* s is free: M^{-1} r for the absolute test */
        rho_old = rho;
        rho = pdot(n, rhat, r);
        rr = pdot(n, r, r);
        mm = pdot(n, s, s);
        conv = BI_DONE(rr, mm);
        if (!conv && omega == 0.0) break;
        if (!conv && rho == 0.0) {
            /* r orthogonal to rhat (e.g. rhat = r0 on the Dirichlet rows only, which the
             * first iteration zeroes): restart the shadow residual, rhat = r, p = v = 0 */
#pragma omp parallel for schedule(static) if (n > PAR_MIN)
            for (int i = 0; i < n; ++i) {
                rhat[i] = r[i];
                p[i] = 0.0;
                v[i] = 0.0;
            }
            rho = rr;
            rho_old = 1.0;
            alpha = 1.0;
            omega = 1.0;
        }
    }
#undef BI_DONE
    if (info) {
        info->iterations = it;
        info->converged = conv;
        info->residual = criterion == 1 ? sqrt(rr) / (bnorm > 0 ? bnorm : 1.0) : sqrt(mm);
    }
    free(w);
    precond_release(&M);
    return conv;
}

/* ------------------------------------------------------- GMRES, CGS2 option */

/* Unrestarted left-preconditioned GMRES as or_gmres (the reference's SolverGMRES),
 * with the Arnoldi vector orthogonalised by classical Gram-Schmidt: h = V^T w,
 * w -= V h, repeated once (h += h2) when ||w|| fell below 0.7 of its norm before the
 * pass.  Stops on |beta_k| < tol; x is updated only on convergence. */
int or_gmres_cgs2(int n, const int* rowptr, const int* col, const double* val, double* x, const double* b,
                  double tol, int maxit, int precond_kind, or_solve_info* info)
{
    if (maxit > n) maxit = n;
    int* st = NULL;
    precond M;
    if (precond_kind == OR_PRECOND_ILU || precond_kind == OR_PRECOND_IC) {
        /* natural order: one row per group */
        st = (int*)malloc(sizeof(int) * (n + 1));
        for (int i = 0; i <= n; ++i) st[i] = i;
    }
    precond_setup(&M, precond_kind, n, rowptr, col, val, st ? n : 0, st);
    double** V = (double**)calloc(maxit + 1, sizeof(double*));
    double* H = (double*)calloc((size_t)(maxit > 0 ? maxit : 1) * (maxit + 1), sizeof(double));
    double* cs = (double*)calloc(maxit + 1, sizeof(double));
    double* sn = (double*)calloc(maxit + 1, sizeof(double));
    double* beta = (double*)calloc(maxit + 2, sizeof(double));
    double* h2 = (double*)calloc(maxit + 1, sizeof(double));
    double* w = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    V[0] = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    or_spmv(n, rowptr, col, val, x, w);
    for (int i = 0; i < n; ++i) w[i] = b[i] - w[i];
    precond_apply(&M, w, V[0]);
    beta[0] = sqrt(pdot(n, V[0], V[0]));
    int it = 0, conv = 0;
    double res = beta[0];
    if (beta[0] < tol) conv = 1;
    else {
        for (int i = 0; i < n; ++i) V[0][i] /= beta[0];
        while (it < maxit) {
            ++it;
            V[it] = (double*)malloc(sizeof(double) * n);
            double* u = V[it];
            or_spmv(n, rowptr, col, val, V[it - 1], w);
            precond_apply(&M, w, u);
            double* h = H + (size_t)(maxit + 1) * (it - 1);
            const double before = sqrt(pdot(n, u, u));
            for (int pass = 0; pass < 2; ++pass) {
                double* c = pass ? h2 : h;
                for (int i = 0; i < it; ++i) c[i] = pdot(n, u, V[i]);
#pragma omp parallel for schedule(static) if (n > PAR_MIN)
                for (int q = 0; q < n; ++q) {
                    double s = u[q];
                    for (int i = 0; i < it; ++i) s -= c[i] * V[i][q];
                    u[q] = s;
                }
                if (pass) for (int i = 0; i < it; ++i) h[i] += h2[i];
                const double after = sqrt(pdot(n, u, u));
                if (pass == 0 && after >= 0.7 * before) break;
            }
            const double aux = sqrt(pdot(n, u, u));
            for (int q = 0; q < n; ++q) u[q] /= aux;
            const int k = it - 1;
            for (int i = 0; i < k; ++i) {
                const double tmp = cs[i] * h[i] + sn[i] * h[i + 1];
                h[i + 1] = -sn[i] * h[i] + cs[i] * h[i + 1];
                h[i] = tmp;
            }
            const double coeff = 1.0 / sqrt(h[k] * h[k] + aux * aux);
            cs[k] = h[k] * coeff;
            sn[k] = aux * coeff;
            h[k] = cs[k] * h[k] + sn[k] * aux;
            beta[k + 1] = -sn[k] * beta[k];
            beta[k] *= cs[k];
            res = fabs(beta[it]);
            if (res < tol) { conv = 1; break; }
        }
        if (conv) {
            double* yv = (double*)malloc(sizeof(double) * it);
            for (int i = it - 1; i >= 0; --i) {
                double s = beta[i];
                for (int j = i + 1; j < it; ++j) s -= H[i + (size_t)(maxit + 1) * j] * yv[j];
                yv[i] = s / H[i + (size_t)(maxit + 1) * i];
            }
            for (int q = 0; q < n; ++q) {
                double s = 0.0;
                for (int j = 0; j < it; ++j) s += V[j][q] * yv[j];
                x[q] += s;
            }
            free(yv);
        }
    }
    if (info) {
        info->iterations = it;
        info->converged = conv;
        info->residual = res;
    }
    for (int k = 0; k <= maxit; ++k) free(V[k]);
    free(V); free(H); free(cs); free(sn); free(beta); free(h2); free(w); free(st);
    precond_release(&M);
    return conv;
}
