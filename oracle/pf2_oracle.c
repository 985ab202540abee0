/*
 * pf2_oracle.c - CPU oracle for the PFEM-2 time-step path (TEST INFRASTRUCTURE ONLY).
 *
 * Single-thread FP64 restatement of the reference gpuPfem2 step path.  Used by the
 * tests, the smoke check and the benchmark's CPU-baseline leg as the checker; never by
 * the product.  Summation orders are deterministic: element order for assembly,
 * particle order for projection, index order for dot products.
 *
 * Known, documented differences from the reference (the reference's results there are
 * timing dependent):
 *  - particle deletion removes exactly the particles that were not found; the
 *    reference's tail-swap (src/particles/particle_handler_2d.cu:164-171) can resurrect
 *    a deleted particle and drop a valid one when holes lie in the tail;
 *  - Dirichlet column elimination decides "skip this row" from the row's first
 *    off-diagonal value before any elimination (the reference reads it while other
 *    threads may be zeroing it, src/Dirichlet_bcs.cu:39-47);
 *  - particle order: the output of or_advect is ordered by cell (stable), reseeded
 *    particles last in each cell in sub-cell order; the reference's order is set by
 *    atomics, so only per-cell multisets are comparable with it.
 */
#include "pf2_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* quadrature: src/integration/quadrature_formula_2d.cu:17-24 (index 1) and
 * src/integration/quadrature_formula_1d.cu:15-18 (index 1).  The tables are the
 * reference's values; z = 1 - x - y is computed as in quadrature_formula_2d.cu:118. */
int or_face_quadrature(int index, double* c3, double* w)
{
    if (index == 0) {
        c3[0] = 0.3333333333333333; c3[1] = 0.3333333333333333;
        c3[2] = 1.0 - c3[0] - c3[1];
        w[0] = 1.0;
        return 1;
    }
    static const double xy[3][2] = {
        { 0.1666666666666667, 0.1666666666666667 },
        { 0.6666666666666667, 0.1666666666666667 },
        { 0.1666666666666667, 0.6666666666666667 } };
    for (int k = 0; k < 3; ++k) {
        c3[3 * k] = xy[k][0];
        c3[3 * k + 1] = xy[k][1];
        c3[3 * k + 2] = 1.0 - xy[k][0] - xy[k][1];
        w[k] = 0.3333333333333333;
    }
    return 3;
}

int or_edge_quadrature(int index, double* c, double* w)
{
    if (index == 0) { c[0] = 0.0; w[0] = 2.0; return 1; }
    c[0] = -0.577350269189626; c[1] = 0.577350269189626;
    w[0] = 1.0; w[1] = 1.0;
    return 2;
}

/* ------------------------------------------------------------------------- */
/* mesh geometry: src/mesh_2d.cu:10-34 (kCalculateCellArea, kCalculateInvJacobi),
 * Matrix2x2::inverse src/common/cuda_math.cuh:124-141.  invJ is stored row-major
 * {d0, d1, d2, d3} = {(0,0), (0,1), (1,0), (1,1)}. */
void or_mesh_geometry(int nc, const double* xy, const int* tri, double* area, double* invJ)
{
    for (int c = 0; c < nc; ++c) {
        const int a = tri[3 * c], b = tri[3 * c + 1], d = tri[3 * c + 2];
        const double v12x = xy[2 * b] - xy[2 * a], v12y = xy[2 * b + 1] - xy[2 * a + 1];
        const double v13x = xy[2 * d] - xy[2 * a], v13y = xy[2 * d + 1] - xy[2 * a + 1];
        /* FMA as nvcc contracts: cross = fma(v12.x, v13.y, -(v12.y * v13.x)) */
        const double cr = fma(v12x, v13y, -(v12y * v13x));
        if (area) area[c] = fabs(cr) * 0.5;
        const double d0 = xy[2 * a] - xy[2 * d], d1 = xy[2 * a + 1] - xy[2 * d + 1];
        const double d2 = xy[2 * b] - xy[2 * d], d3 = xy[2 * b + 1] - xy[2 * d + 1];
        const double det = fma(d0, d3, -(d1 * d2));
        const double invdet = 1.0 / det;
        if (invJ) {
            invJ[4 * c + 0] = d3 * invdet;
            invJ[4 * c + 1] = -d1 * invdet;
            invJ[4 * c + 2] = -d2 * invdet;
            invJ[4 * c + 3] = d0 * invdet;
        }
    }
}

static int cmp_int(const void* a, const void* b)
{
    const int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}

/* node -> incident cells (ascending), the incidence used below */
int or_node_cells(int nv, int nc, const int* tri, int* off, int* cells)
{
    memset(off, 0, sizeof(int) * (nv + 1));
    for (int c = 0; c < nc; ++c)
        for (int k = 0; k < 3; ++k) off[tri[3 * c + k] + 1]++;
    for (int i = 0; i < nv; ++i) off[i + 1] += off[i];
    if (cells) {
        int* fill = (int*)malloc(sizeof(int) * nv);
        memcpy(fill, off, sizeof(int) * nv);
        for (int c = 0; c < nc; ++c)
            for (int k = 0; k < 3; ++k) cells[fill[tri[3 * c + k]]++] = c; /* ascending c */
        free(fill);
    }
    return off[nv];
}

/* Cells sharing at least one vertex with a cell, ascending, without the cell itself:
 * the set the reference builds with its all-pairs loop (src/mesh_2d.cu:107-139),
 * computed here from the node incidence. */
int or_neighbors(int nv, int nc, const int* tri, int* off, int* idx)
{
    int* noff = (int*)malloc(sizeof(int) * (nv + 1));
    const int ninc = or_node_cells(nv, nc, tri, noff, NULL);
    int* ncell = (int*)malloc(sizeof(int) * (ninc > 0 ? ninc : 1));
    or_node_cells(nv, nc, tri, noff, ncell);
    int buf[1024];
    int total = 0;
    off[0] = 0;
    for (int c = 0; c < nc; ++c) {
        int m = 0;
        for (int k = 0; k < 3; ++k) {
            const int v = tri[3 * c + k];
            for (int q = noff[v]; q < noff[v + 1]; ++q)
                if (ncell[q] != c && m < 1024) buf[m++] = ncell[q];
        }
        qsort(buf, m, sizeof(int), cmp_int);
        int u = 0;
        for (int q = 0; q < m; ++q)
            if (q == 0 || buf[q] != buf[q - 1]) {
                if (idx) idx[total + u] = buf[q];
                ++u;
            }
        total += u;
        off[c + 1] = total;
    }
    free(noff);
    free(ncell);
    return total;
}

/* CSR structure: rows = nodes, columns = {i} U {vertices of incident triangles},
 * ascending (src/linear_algebra/sparse_matrix.cu:8-54). */
int or_csr_structure(int nv, int nc, const int* tri, int* rowptr, int* col)
{
    int* noff = (int*)malloc(sizeof(int) * (nv + 1));
    const int ninc = or_node_cells(nv, nc, tri, noff, NULL);
    int* ncell = (int*)malloc(sizeof(int) * (ninc > 0 ? ninc : 1));
    or_node_cells(nv, nc, tri, noff, ncell);
    int buf[1024];
    int total = 0;
    rowptr[0] = 0;
    for (int i = 0; i < nv; ++i) {
        int m = 0;
        buf[m++] = i;
        for (int q = noff[i]; q < noff[i + 1]; ++q)
            for (int k = 0; k < 3; ++k)
                if (m < 1024) buf[m++] = tri[3 * ncell[q] + k];
        qsort(buf, m, sizeof(int), cmp_int);
        int u = 0;
        for (int q = 0; q < m; ++q)
            if (q == 0 || buf[q] != buf[q - 1]) {
                if (col) col[total + u] = buf[q];
                ++u;
            }
        total += u;
        rowptr[i + 1] = total;
    }
    free(noff);
    free(ncell);
    return total;
}

/* Edge boundary ids of the channel drivers (cases/Cylinder2D/main.cu:35-70):
 * edge i of a cell runs from vertex i to vertex (i+1)%3; its midpoint decides
 * 0 inlet (x=0), 1 outlet (x=lx), 2 walls (y=0, y=ly), 3 cylinder (|d - r| < 0.001). */
void or_edge_boundary_ids(int nc, const double* xy, const int* tri, double lx, double ly,
                          int has_cyl, double cx, double cy, double r, int* ids3)
{
    for (int c = 0; c < nc; ++c)
        for (int i = 0; i < 3; ++i) {
            const int s = tri[3 * c + i], e = tri[3 * c + (i + 1) % 3];
            const double mx = (xy[2 * s] + xy[2 * e]) * 0.5;
            const double my = (xy[2 * s + 1] + xy[2 * e + 1]) * 0.5;
            int id = -1;
            if (fabs(mx) < OR_DOUBLE_MIN) id = 0;
            else if (fabs(mx - lx) < OR_DOUBLE_MIN) id = 1;
            else if (fabs(my) < OR_DOUBLE_MIN || fabs(my - ly) < OR_DOUBLE_MIN) id = 2;
            else if (has_cyl) {
                const double dx = mx - cx, dy = my - cy;
                if (fabs(sqrt(dx * dx + dy * dy) - r) < 0.001) id = 3;
            }
            ids3[3 * c + i] = id;
        }
}

/* ------------------------------------------------------------------------- */
int or_find_in_row(const int* rowptr, const int* col, int row, int target)
{
    int lo = rowptr[row], hi = rowptr[row + 1] - 1;
    while (lo <= hi) {
        const int m = (lo + hi) >> 1;
        if (col[m] == target) return m;
        if (col[m] < target) lo = m + 1; else hi = m - 1;
    }
    return -1;
}

void or_spmv(int n, const int* rowptr, const int* col, const double* val, const double* x, double* y)
{
    /* rows are independent: the threads change no bits */
#pragma omp parallel for schedule(static) if (n > 65536)
    for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) s += val[k] * x[col[k]];
        y[i] = s;
    }
}

/* addLocalToGlobal (src/integration/numerical_integrator_2d.cuh:22-43) */
static void add_local(const int* t, double area, const double M[3][3], const double R[3],
                      const int* rowptr, const int* col, double* val, double* rhs)
{
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) {
            const int k = or_find_in_row(rowptr, col, t[i], t[j]);
            if (k >= 0) val[k] += M[i][j] * area;
        }
        rhs[t[i]] += R[i] * area;
    }
}

/* invJ * shapeFuncGrad(i) (numerical_integrator_2d.cuh:8-20, cuda_math.cuh:146-153) */
static void shape_grad(const double* J, int i, double* g)
{
    static const double sg[3][2] = { { 1.0, 0.0 }, { 0.0, 1.0 }, { -1.0, -1.0 } };
    g[0] = J[0] * sg[i][0] + J[1] * sg[i][1];
    g[1] = J[2] * sg[i][0] + J[3] * sg[i][1];
}

static double rhs_function(int kind, double x, double y)
{
    if (kind == OR_RHS_SINSIN) {
        const double pi = 3.14159265358979323846;
        return 2.0 * pi * pi * sin(pi * x) * sin(pi * y);
    }
    return exp(-(x * x + 10 * y * y)); /* cases/Poisson2D/main.cu:24-26 */
}

/* Poisson assembly, cases/Poisson2D/main.cu:28-68 (lambda and the right-hand side
 * are parameters; the shipped case uses lambda = 0.5 and exp(-(x^2+10y^2))). */
void or_assemble_poisson(int nc, const double* xy, const int* tri, const double* area, const double* invJ,
                         int rhs_kind, double lambda, const int* rowptr, const int* col, double* val, double* rhs)
{
    double qc[9], qw[3];
    const int nq = or_face_quadrature(1, qc, qw);
    for (int c = 0; c < nc; ++c) {
        const int* t = tri + 3 * c;
        const double* J = invJ + 4 * c;
        double M[3][3] = { { 0 } }, R[3] = { 0 };
        for (int q = 0; q < nq; ++q) {
            const double* L = qc + 3 * q;
            const double px = L[0] * xy[2 * t[0]] + L[1] * xy[2 * t[1]] + L[2] * xy[2 * t[2]];
            const double py = L[0] * xy[2 * t[0] + 1] + L[1] * xy[2 * t[1] + 1] + L[2] * xy[2 * t[2] + 1];
            const double f = rhs_function(rhs_kind, px, py);
            for (int i = 0; i < 3; ++i) {
                double gi[2];
                shape_grad(J, i, gi);
                for (int j = i; j < 3; ++j) {
                    double gj[2];
                    shape_grad(J, j, gj);
                    const double aux = lambda * (gi[0] * gj[0] + gi[1] * gj[1]) * qw[q];
                    M[i][j] += aux;
                    if (j != i) M[j][i] = M[i][j];
                }
                R[i] += f * L[i] * qw[q];
            }
        }
        add_local(t, area[c], M, R, rowptr, col, val, rhs);
    }
}

/* ------------------------------------------------------------------------- */
/* Dirichlet BCs, src/Dirichlet_bcs.cu:3-51 and :73-86: boundary rows become e_i with
 * rhs g; for every other row r that couples to a boundary node d, rhs_r -= a_rd g_d and
 * a_rd = 0, unless |first off-diagonal of row r| < 2e-6 (the reference's test for
 * "row r is another boundary row"), read before any elimination. */
void or_apply_bcs(int n, const int* rowptr, const int* col, double* val, double* rhs,
                  int nbc, const int* bc_node, const double* bc_val)
{
    for (int b = 0; b < nbc; ++b) {
        const int d = bc_node[b];
        for (int k = rowptr[d]; k < rowptr[d + 1]; ++k) val[k] = (col[k] == d) ? 1.0 : 0.0;
        rhs[d] = bc_val[b];
    }
    unsigned char* skip = (unsigned char*)calloc(n > 0 ? n : 1, 1);
    for (int r = 0; r < n; ++r) {
        const int s = rowptr[r];
        const int first = s + (col[s] == r);
        /* a row holding only its diagonal has no off-diagonal entry: nothing to skip on */
        skip[r] = (first < rowptr[n]) ? (fabs(val[first]) < OR_DOUBLE_MIN) : 1;
    }
    for (int b = 0; b < nbc; ++b) {
        const int d = bc_node[b];
        const double mg = -bc_val[b];
        for (int k = rowptr[d]; k < rowptr[d + 1]; ++k) {
            const int r = col[k];
            if (r == d || skip[r]) continue;
            const int q = or_find_in_row(rowptr, col, r, d);
            if (q >= 0) {
                rhs[r] += val[q] * mg;
                val[q] = 0.0;
            }
        }
    }
    free(skip);
}

/* ------------------------------------------------------------------------- */
/* Preconditioners, src/linear_algebra/preconditioners.cu: Jacobi (:3-46), ILU(0)
 * (:48-134, cusparseDcsrilu02: zero-fill ILU, unit L / non-unit U on one CSR copy)
 * and IC(0) (:136-213, cusparseDcsric02: lower L with A ~ L L^T).  The
 * factorisations are restated from their standard zero-fill definitions (Saad,
 * Iterative Methods for Sparse Linear Systems, Alg. 10.4 and the IC(0) analogue). */
static int diag_pos(const int* rowptr, const int* col, int i) { return or_find_in_row(rowptr, col, i, i); }

void or_ilu0(int n, const int* rowptr, const int* col, double* a)
{
    for (int i = 0; i < n; ++i) {
        for (int kk = rowptr[i]; kk < rowptr[i + 1] && col[kk] < i; ++kk) {
            const int k = col[kk];
            a[kk] = a[kk] / a[diag_pos(rowptr, col, k)];
            for (int jj = kk + 1; jj < rowptr[i + 1]; ++jj) {
                const int q = or_find_in_row(rowptr, col, k, col[jj]);
                if (q >= 0) a[jj] -= a[kk] * a[q];
            }
        }
    }
}

void or_ic0(int n, const int* rowptr, const int* col, double* l)
{
    for (int i = 0; i < n; ++i) {
        const int s = rowptr[i];
        int e = s;
        while (e < rowptr[i + 1] && col[e] < i) ++e; /* [s, e) strictly lower, e = diagonal */
        for (int kk = s; kk < e; ++kk) {
            const int k = col[kk];
            /* sum_{j<k} l_ij l_kj over the common lower pattern */
            double sum = l[kk];
            int p = s, q = rowptr[k];
            while (p < kk && q < rowptr[k + 1] && col[q] < k) {
                if (col[p] == col[q]) { sum -= l[p] * l[q]; ++p; ++q; }
                else if (col[p] < col[q]) ++p;
                else ++q;
            }
            l[kk] = sum / l[diag_pos(rowptr, col, k)];
        }
        double d = l[e];
        for (int kk = s; kk < e; ++kk) d -= l[kk] * l[kk];
        l[e] = sqrt(d);
    }
}

void or_precond_apply(int kind, int n, const int* rowptr, const int* col, const double* f,
                      const double* invdiag, const double* src, double* dst, double* tmp)
{
    if (kind == OR_PRECOND_NONE) { memmove(dst, src, sizeof(double) * n); return; }
    if (kind == OR_PRECOND_JACOBI) {
        for (int i = 0; i < n; ++i) dst[i] = src[i] * invdiag[i];
        return;
    }
    /* forward solve with the lower factor (unit for ILU, l_ii for IC) */
    for (int i = 0; i < n; ++i) {
        double s = src[i];
        int k = rowptr[i];
        for (; k < rowptr[i + 1] && col[k] < i; ++k) s -= f[k] * tmp[col[k]];
        tmp[i] = (kind == OR_PRECOND_IC) ? s / f[k] : s;
    }
    if (kind == OR_PRECOND_ILU) {
        for (int i = n - 1; i >= 0; --i) {
            double s = tmp[i];
            const int d = diag_pos(rowptr, col, i);
            for (int k = d + 1; k < rowptr[i + 1]; ++k) s -= f[k] * dst[col[k]];
            dst[i] = s / f[d];
        }
    } else {
        /* L^T z = y, column sweep over the rows of L */
        for (int i = 0; i < n; ++i) dst[i] = tmp[i];
        for (int i = n - 1; i >= 0; --i) {
            const int d = diag_pos(rowptr, col, i);
            dst[i] = dst[i] / f[d];
            for (int k = rowptr[i]; k < d; ++k) dst[col[k]] -= f[k] * dst[i];
        }
    }
}

typedef struct {
    int kind;
    double* fact;
    double* invdiag;
    double* tmp;
} or_precond;

static void precond_init(or_precond* P, int kind, int n, const int* rowptr, const int* col, const double* val)
{
    P->kind = kind;
    P->fact = NULL;
    P->invdiag = NULL;
    P->tmp = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
    if (kind == OR_PRECOND_JACOBI) {
        P->invdiag = (double*)malloc(sizeof(double) * n);
        for (int i = 0; i < n; ++i) {
            const int d = diag_pos(rowptr, col, i);
            P->invdiag[i] = (d >= 0) ? 1.0 / val[d] : 0.0;
        }
    } else if (kind == OR_PRECOND_ILU || kind == OR_PRECOND_IC) {
        const int nnz = rowptr[n];
        P->fact = (double*)malloc(sizeof(double) * nnz);
        memcpy(P->fact, val, sizeof(double) * nnz);
        if (kind == OR_PRECOND_ILU) or_ilu0(n, rowptr, col, P->fact);
        else or_ic0(n, rowptr, col, P->fact);
    }
}

static void precond_free(or_precond* P)
{
    free(P->fact);
    free(P->invdiag);
    free(P->tmp);
}

/* Dot product summed over fixed 4,096-entry chunks in chunk order: the bits do not
 * depend on the number of threads. */
static double dotv(int n, const double* a, const double* b)
{
    enum { CH = 4096 };
    const int nch = (n + CH - 1) / CH;
    double stack[256];
    double* part = nch <= 256 ? stack : (double*)malloc(sizeof(double) * nch);
#pragma omp parallel for schedule(static) if (n > 32768)
    for (int c = 0; c < nch; ++c) {
        const int i1 = (c + 1) * CH < n ? (c + 1) * CH : n;
        double s = 0.0;
        for (int i = c * CH; i < i1; ++i) s += a[i] * b[i];
        part[c] = s;
    }
    double s = 0.0;
    for (int c = 0; c < nch; ++c) s += part[c];
    if (part != stack) free(part);
    return s;
}

/* Preconditioned CG, SolverCG::solve src/linear_algebra/linear_solver.cu:440-515:
 * x0 is the incoming x; stop when r^T z < tol^2 (absolute), at most maxit iterations. */
int or_pcg(int n, const int* rowptr, const int* col, const double* val, double* x, const double* b,
           double tol, int maxit, int precond, or_solve_info* info)
{
    or_precond P;
    precond_init(&P, precond, n, rowptr, col, val);
    double* r = (double*)malloc(sizeof(double) * n);
    double* z = (double*)malloc(sizeof(double) * n);
    double* p = (double*)malloc(sizeof(double) * n);
    double* q = (double*)malloc(sizeof(double) * n);
    or_spmv(n, rowptr, col, val, x, q);
    for (int i = 0; i < n; ++i) r[i] = b[i] - q[i];
    or_precond_apply(precond, n, rowptr, col, P.fact, P.invdiag, r, z, P.tmp);
    memcpy(p, z, sizeof(double) * n);
    double gamma = dotv(n, r, z);
    const double tol2 = tol * tol;
    int it = 0, conv = 0;
    if (gamma < tol2) conv = 1;
    while (!conv && it < maxit) {
        ++it;
        or_spmv(n, rowptr, col, val, p, q);
        const double pq = dotv(n, p, q);
        for (int i = 0; i < n; ++i) {
            const double alpha = gamma / pq;
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        or_precond_apply(precond, n, rowptr, col, P.fact, P.invdiag, r, z, P.tmp);
        const double gold = gamma;
        gamma = dotv(n, r, z);
        if (gamma < tol2) { conv = 1; break; }
        for (int i = 0; i < n; ++i) {
            const double beta = gamma / gold;
            p[i] = z[i] + beta * p[i];
        }
    }
    if (info) {
        info->iterations = it;
        info->converged = conv;
        info->residual = sqrt(gamma);
    }
    free(r); free(z); free(p); free(q);
    precond_free(&P);
    return conv;
}

/* GMRES without restart, SolverGMRES::solve src/linear_algebra/linear_solver.cu:560-660:
 * left preconditioning, Gram-Schmidt as the reference runs it (each projection uses
 * the already-updated vector), Givens rotations (updateHcolumn :40-66), stop on
 * |beta_k| < tol; x is updated only on convergence. */
int or_gmres(int n, const int* rowptr, const int* col, const double* val, double* x, const double* b,
             double tol, int maxit, int precond, or_solve_info* info)
{
    if (maxit > n) maxit = n; /* SolverGMRES::init clamps (linear_solver.cu:396-399) */
    or_precond P;
    precond_init(&P, precond, n, rowptr, col, val);
    int vcap = 8;
    double** V = (double**)malloc(sizeof(double*) * (maxit + 1));
    for (int k = 0; k <= maxit; ++k) V[k] = NULL;
    double* H = (double*)calloc((size_t)maxit * (maxit > 0 ? maxit : 1), sizeof(double));
    double* cs = (double*)calloc(maxit + 1, sizeof(double));
    double* sn = (double*)calloc(maxit + 1, sizeof(double));
    double* beta = (double*)calloc(maxit + 2, sizeof(double));
    (void)vcap;
    V[0] = (double*)malloc(sizeof(double) * n);
    double* w = (double*)malloc(sizeof(double) * n);
    or_spmv(n, rowptr, col, val, x, w);
    for (int i = 0; i < n; ++i) w[i] = b[i] - w[i];
    or_precond_apply(precond, n, rowptr, col, P.fact, P.invdiag, w, V[0], P.tmp);
    beta[0] = sqrt(dotv(n, V[0], V[0]));
    int it = 0, conv = 0;
    double res = beta[0];
    if (beta[0] < tol) conv = 1;
    else {
        for (int i = 0; i < n; ++i) V[0][i] = V[0][i] / beta[0];
        while (it < maxit) {
            ++it;
            V[it] = (double*)malloc(sizeof(double) * n);
            double* vk = V[it - 1];
            double* vkp = V[it];
            or_spmv(n, rowptr, col, val, vk, w);
            or_precond_apply(precond, n, rowptr, col, P.fact, P.invdiag, w, vkp, P.tmp);
            double* h = H + (size_t)maxit * (it - 1);
            for (int i = 0; i < it; ++i) {
                h[i] = dotv(n, vkp, V[i]);
                const double hi = h[i];
                const double* vi = V[i];
#pragma omp parallel for schedule(static) if (n > 32768)
                for (int q = 0; q < n; ++q) vkp[q] -= hi * vi[q];
            }
            double aux = sqrt(dotv(n, vkp, vkp));
            for (int q = 0; q < n; ++q) vkp[q] = vkp[q] / aux;
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
            /* y = H^{-1} beta (upper triangular, column-major lda = maxit), x += V y */
            double* y = (double*)malloc(sizeof(double) * it);
            for (int i = it - 1; i >= 0; --i) {
                double s = beta[i];
                for (int j = i + 1; j < it; ++j) s -= H[i + (size_t)maxit * j] * y[j];
                y[i] = s / H[i + (size_t)maxit * i];
            }
            for (int q = 0; q < n; ++q) {
                double s = 0.0;
                for (int j = 0; j < it; ++j) s += V[j][q] * y[j];
                x[q] = s + x[q];
            }
            free(y);
        }
    }
    if (info) {
        info->iterations = it;
        info->converged = conv;
        info->residual = res;
    }
    for (int k = 0; k <= maxit; ++k) free(V[k]);
    free(V); free(H); free(cs); free(sn); free(beta); free(w);
    precond_free(&P);
    return conv;
}

/* ------------------------------------------------------------------------- */
/* Particles. */

/* Sub-triangle centroids, ParticleHandler2D::ParticleHandler2D
 * src/particles/particle_handler_2d.cu:238-294; level clamped to [1, 4]. */
int or_subcell_centers(int level, double* c3)
{
    const int n = level < 1 ? 1 : (level > OR_MAX_LEVEL ? OR_MAX_LEVEL : level);
    const double dx = 1.0 / n;
    int k = 0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < 2 * i + 1; ++j) {
            const double xmin = (j / 2) * dx, xmax = xmin + dx;
            const double ymin = (n - 1 - i) * dx, ymax = ymin + dx;
            double v0[3] = { xmin, ymax, 1.0 - xmin - ymax };
            double v1[3];
            v1[0] = (j % 2 == 0) ? xmin : xmax;
            v1[1] = (j % 2 == 0) ? ymin : ymax;
            v1[2] = 1.0 - v1[0] - v1[1];
            double v2[3] = { xmax, ymin, 1.0 - xmax - ymin };
            for (int a = 0; a < 3; ++a) c3[3 * k + a] = 0.3333333333333333 * ((v0[a] + v1[a]) + v2[a]);
            ++k;
        }
    return n;
}

/* determineSubcell, src/particles/particle_handler_2d.cu:10-33 (no clamping: an
 * index >= level^2 addresses the following cell, as in the reference). */
int or_determine_subcell(int n, double step, const double* l)
{
    int res = 0;
    const int i = (int)((1.0 - l[1]) * (double)n);
    for (int row = 0; row < i; ++row) res += 2 * row + 1;
    const int j = (int)(l[0] * (double)n);
    res += 2 * j;
    if (j != i) {
        const double x = step * (double)(j + 1);
        const double y = fma(-step, (double)(i + 1), 1.0); /* FMA as nvcc contracts */
        const double z = 1.0 - x - y;
        if (l[2] < z) ++res;
    }
    return res;
}

/* transformLocalToGlobal (geometry.cuh:6-8), FMA as nvcc contracts */
static void local_to_global(const double* L, const double* xy, const int* t, double* p)
{
    for (int a = 0; a < 2; ++a)
        p[a] = fma(xy[2 * t[2] + a], L[2], fma(xy[2 * t[0] + a], L[0], xy[2 * t[1] + a] * L[1]));
}

/* sum_i L_i u(node_i), accumulated from 0.0 as the reference's loops do
 * (particle_handler_2d.cu:62-66, :224-227), FMA as nvcc contracts */
static double interp(const double* L, const int* t, const double* u)
{
    double s = fma(L[0], u[t[0]], 0.0);
    s = fma(L[1], u[t[1]], s);
    s = fma(L[2], u[t[2]], s);
    return s;
}

/* kSeedParticlesIntoCell, particle_handler_2d.cu:35-52: cell-major order here. */
int or_seed(int nc, const double* xy, const int* tri, int level, const double* c3,
            double* px, double* py, double* l0, double* l1, double* l2, double* pu, double* pv, int* cell)
{
    const int ppc = level * level;
    for (int c = 0; c < nc; ++c)
        for (int k = 0; k < ppc; ++k) {
            const int p = c * ppc + k;
            double pos[2];
            local_to_global(c3 + 3 * k, xy, tri + 3 * c, pos);
            px[p] = pos[0]; py[p] = pos[1];
            l0[p] = c3[3 * k]; l1[p] = c3[3 * k + 1]; l2[p] = c3[3 * k + 2];
            pu[p] = 0.0; pv[p] = 0.0;
            cell[p] = c;
        }
    return nc * ppc;
}

/* Global -> local and the inside test: Particle2D::isInsideCell particle_2d.cu:14-22,
 * GEOMETRY::transformGlobalToLocal geometry.cuh:14-23, isPointInsideUnitTriangle
 * geometry.cuh:37-46.  Returns 1 and writes l3 when inside. */
static int inside_cell(double x, double y, int c, const double* xy, const int* tri, const double* invJ, double* l3)
{
    const int v = tri[3 * c + 2];
    const double dx = x - xy[2 * v], dy = y - xy[2 * v + 1];
    const double* J = invJ + 4 * c;
    const double lx = fma(J[0], dx, J[2] * dy); /* FMA as nvcc contracts */
    const double ly = fma(J[1], dx, J[3] * dy);
    const double lz = 1.0 - lx - ly;
    const double hi = 1.0 + OR_DOUBLE_MIN, lo = -OR_DOUBLE_MIN;
    if (lx > hi || lx < lo) return 0;
    if (ly > hi || ly < lo) return 0;
    if (lz > hi || lz < lo) return 0;
    l3[0] = lx; l3[1] = ly; l3[2] = lz;
    return 1;
}

/* Cell location after a move: own cell first (kCheckParticleInCell :117-131), then the
 * vertex-sharing neighbours in ascending order, first hit wins (kCheckParticleInNeighbors
 * :133-162).  Returns the cell or -1 (deleted). */
int or_locate(double x, double y, int c, const double* xy, const int* tri, const double* invJ,
              const int* nb_off, const int* nb_idx, double* l3)
{
    if (inside_cell(x, y, c, xy, tri, invJ, l3)) return c;
    for (int k = nb_off[c]; k < nb_off[c + 1]; ++k)
        if (inside_cell(x, y, nb_idx[k], xy, tri, invJ, l3)) return nb_idx[k];
    return -1;
}

/* ParticleHandler2D::advectParticles (:328-342) with kAdvectParticles (:54-70), the
 * location of sortParticlesInCells (:363-395) after each substep, and
 * checkParticleDistribution (:397-423) with kCountParticlesInSubcells (:173-181) and
 * kAddParticlesToCell (:197-236). */
int or_advect(int np, int cap, double* px, double* py, double* l0, double* l1, double* l2,
              double* pu, double* pv, int* cell,
              int nv, const double* xy, int nc, const int* tri, const double* invJ,
              const int* nb_off, const int* nb_idx, const double* ux, const double* uy,
              double dt, int substeps, int level, const double* c3, int* n_deleted, int* n_added)
{
    (void)nv;
    const double dts = dt / substeps;
    int deleted = 0;
    /* particles are independent: the threads change no bits */
#pragma omp parallel for schedule(static) reduction(+ : deleted) if (np > 65536)
    for (int p = 0; p < np; ++p) {
        int c = cell[p];
        double L[3] = { l0[p], l1[p], l2[p] };
        double x = px[p], y = py[p];
        for (int s = 0; s < substeps && c >= 0; ++s) {
            const int* t = tri + 3 * c;
            const double vx = interp(L, t, ux), vy = interp(L, t, uy);
            x = fma(vx, dts, x);
            y = fma(vy, dts, y);
            double Ln[3];
            const int cn = or_locate(x, y, c, xy, tri, invJ, nb_off, nb_idx, Ln);
            if (cn < 0) { c = -1; break; }
            c = cn;
            L[0] = Ln[0]; L[1] = Ln[1]; L[2] = Ln[2];
        }
        px[p] = x; py[p] = y;
        l0[p] = L[0]; l1[p] = L[1]; l2[p] = L[2];
        cell[p] = c;
        if (c < 0) ++deleted;
    }
    /* population of the sub-cells */
    const int ppc = level * level;
    const double step = 1.0 / level;
    const long long nsub = (long long)nc * ppc;
    int* cnt = (int*)calloc(nsub > 0 ? nsub : 1, sizeof(int));
    int* percell = (int*)calloc(nc + 1, sizeof(int));
    for (int p = 0; p < np; ++p) {
        if (cell[p] < 0) continue;
        const double L[3] = { l0[p], l1[p], l2[p] };
        const long long g = (long long)cell[p] * ppc + or_determine_subcell(level, step, L);
        if (g < nsub) cnt[g]++;
        percell[cell[p]]++;
    }
    int added = 0;
    for (long long g = 0; g < nsub; ++g) added += (cnt[g] == 0);
    const int nnew = np - deleted + added;
    if (n_deleted) *n_deleted = deleted;
    if (n_added) *n_added = added;
    if (nnew > cap) { free(cnt); free(percell); return -1; }
    /* stable counting sort by cell, reseeded particles appended per cell */
    int* start = (int*)malloc(sizeof(int) * (nc + 1));
    start[0] = 0;
    for (int c = 0; c < nc; ++c) {
        int add = 0;
        for (int k = 0; k < ppc; ++k) add += (cnt[(long long)c * ppc + k] == 0);
        start[c + 1] = start[c] + percell[c] + add;
    }
    double* bx = (double*)malloc(sizeof(double) * (nnew > 0 ? nnew : 1) * 7);
    double *by = bx + nnew, *b0 = by + nnew, *b1 = b0 + nnew, *b2 = b1 + nnew, *bu = b2 + nnew, *bv = bu + nnew;
    int* bc = (int*)malloc(sizeof(int) * (nnew > 0 ? nnew : 1));
    int* fill = (int*)malloc(sizeof(int) * (nc + 1));
    memcpy(fill, start, sizeof(int) * (nc + 1));
    for (int p = 0; p < np; ++p) {
        const int c = cell[p];
        if (c < 0) continue;
        const int o = fill[c]++;
        bx[o] = px[p]; by[o] = py[p]; b0[o] = l0[p]; b1[o] = l1[p]; b2[o] = l2[p];
        bu[o] = pu[p]; bv[o] = pv[p]; bc[o] = c;
    }
    for (int c = 0; c < nc; ++c)
        for (int k = 0; k < ppc; ++k) {
            if (cnt[(long long)c * ppc + k] != 0) continue;
            const int o = fill[c]++;
            const int* t = tri + 3 * c;
            double pos[2];
            local_to_global(c3 + 3 * k, xy, t, pos);
            bx[o] = pos[0]; by[o] = pos[1];
            b0[o] = c3[3 * k]; b1[o] = c3[3 * k + 1]; b2[o] = c3[3 * k + 2];
            bu[o] = interp(c3 + 3 * k, t, ux);
            bv[o] = interp(c3 + 3 * k, t, uy);
            bc[o] = c;
        }
    memcpy(px, bx, sizeof(double) * nnew); memcpy(py, by, sizeof(double) * nnew);
    memcpy(l0, b0, sizeof(double) * nnew); memcpy(l1, b1, sizeof(double) * nnew);
    memcpy(l2, b2, sizeof(double) * nnew); memcpy(pu, bu, sizeof(double) * nnew);
    memcpy(pv, bv, sizeof(double) * nnew); memcpy(cell, bc, sizeof(int) * nnew);
    free(bx); free(bc); free(fill); free(start); free(cnt); free(percell);
    return nnew;
}

/* kProjectParticleVelocityOntoGrid (:90-107) + kFinalizeVelocityProjection (:109-115):
 * u_node = sum_p L_i v_p / sum_p L_i, accumulated in particle order. */
void or_project(int np, const int* tri, const int* cell, const double* l0, const double* l1, const double* l2,
                const double* pu, const double* pv, int nv, double* ux, double* uy)
{
    double* w = (double*)calloc(nv, sizeof(double));
    double* sx = (double*)calloc(nv, sizeof(double));
    double* sy = (double*)calloc(nv, sizeof(double));
    for (int p = 0; p < np; ++p) {
        const int* t = tri + 3 * cell[p];
        const double L[3] = { l0[p], l1[p], l2[p] };
        for (int i = 0; i < 3; ++i) {
            sx[t[i]] += L[i] * pu[p];
            sy[t[i]] += L[i] * pv[p];
            w[t[i]] += L[i];
        }
    }
    for (int i = 0; i < nv; ++i) {
        ux[i] = sx[i] / w[i];
        uy[i] = sy[i] / w[i];
    }
    free(w); free(sx); free(sy);
}

/* kCorrectParticleVelocity (:72-88): v_p += sum_i L_i (u_i - u_old_i); with no old
 * field (initParticleVelocity, :322-326) the increment is sum_i L_i u_i. */
void or_correct_velocity(int np, const int* tri, const int* cell, const double* l0, const double* l1,
                         const double* l2, const double* ux, const double* uy,
                         const double* ux_old, const double* uy_old, double* pu, double* pv)
{
    for (int p = 0; p < np; ++p) {
        const int* t = tri + 3 * cell[p];
        const double L[3] = { l0[p], l1[p], l2[p] };
        double ix = 0.0, iy = 0.0;
        for (int i = 0; i < 3; ++i) {
            const double dx = ux[t[i]] - (ux_old ? ux_old[t[i]] : 0.0);
            const double dy = uy[t[i]] - (uy_old ? uy_old[t[i]] : 0.0);
            ix = fma(L[i], dx, ix); /* FMA as nvcc contracts */
            iy = fma(L[i], dy, iy);
        }
        pu[p] = pu[p] + ix;
        pv[p] = pv[p] + iy;
    }
}

/* ------------------------------------------------------------------------- */
/* Flow assembly, cases/Cylinder2D/main.cu. */

/* kIntegrateVelocityPrediction :72-167 (outlet edge term on boundary id 1, n = (1,0);
 * like the cell terms, it is multiplied by the cell area in addLocalToGlobal). */
void or_assemble_prediction(int nc, const double* xy, const int* tri, const double* area, const double* invJ,
                            const int* edge_ids, const or_params* P, const double* ux, const double* uy,
                            const double* ux_old, const double* uy_old, const double* p_old,
                            const int* rowptr, const int* col, double* val_x, double* val_y,
                            double* rhs_x, double* rhs_y)
{
    double qc[9], qw[3], ec[2], ew[2];
    const int nq = or_face_quadrature(1, qc, qw);
    const int ne = or_edge_quadrature(1, ec, ew);
    const double* u[2] = { ux, uy };
    const double* uo[2] = { ux_old, uy_old };
    for (int c = 0; c < nc; ++c) {
        const int* t = tri + 3 * c;
        const double* J = invJ + 4 * c;
        double M[2][3][3] = { { { 0 } } }, R[2][3] = { { 0 } };
        for (int q = 0; q < nq; ++q) {
            const double* L = qc + 3 * q;
            for (int i = 0; i < 3; ++i) {
                double gi[2];
                shape_grad(J, i, gi);
                const double Ni = L[i];
                for (int j = 0; j < 3; ++j) {
                    double gj[2];
                    shape_grad(J, j, gj);
                    const double Nj = L[j];
                    double aux = P->rho * Ni * Nj * qw[q];
                    for (int k = 0; k < 2; ++k) {
                        M[k][i][j] += aux;
                        R[k][i] += aux * uo[k][t[j]];
                    }
                    aux = P->mu * P->dt * qw[q];
                    M[0][i][j] += aux * (gi[1] * gj[1] + 4.0 / 3.0 * gi[0] * gj[0]);
                    M[1][i][j] += aux * (gi[0] * gj[0] + 4.0 / 3.0 * gi[1] * gj[1]);
                    R[0][i] -= aux * (gi[1] * gj[0] - 2.0 / 3.0 * gi[0] * gj[1]) * u[1][t[j]];
                    R[1][i] -= aux * (gi[0] * gj[1] - 2.0 / 3.0 * gi[1] * gj[0]) * u[0][t[j]];
                    if (p_old) {
                        aux = Ni * p_old[t[j]] * P->dt * qw[q];
                        R[0][i] -= aux * gj[0];
                        R[1][i] -= aux * gj[1];
                    }
                }
            }
        }
        for (int e = 0; e < 3; ++e) {
            if (edge_ids[3 * c + e] != 1) continue;
            const double nx = 1.0, ny = 0.0;
            const int s = t[e], f = t[(e + 1) % 3];
            const double sx = xy[2 * s], sy = xy[2 * s + 1], fx = xy[2 * f], fy = xy[2 * f + 1];
            const double half = 0.5 * sqrt((sx - fx) * (sx - fx) + (sy - fy) * (sy - fy));
            for (int q = 0; q < ne; ++q) {
                const double qx = 0.5 * (ec[q] * (fx - sx) + (sx + fx));
                const double qy = 0.5 * (ec[q] * (fy - sy) + (sy + fy));
                const int v3 = t[2];
                const double dx = qx - xy[2 * v3], dy = qy - xy[2 * v3 + 1];
                double L[3];
                L[0] = J[0] * dx + J[2] * dy;
                L[1] = J[1] * dx + J[3] * dy;
                L[2] = 1.0 - L[0] - L[1];
                const double aux = P->mu * P->dt * ew[q] * half;
                for (int i = 0; i < 3; ++i) {
                    const double Ni = L[i];
                    for (int j = 0; j < 3; ++j) {
                        double gj[2];
                        shape_grad(J, j, gj);
                        M[0][i][j] -= aux * Ni * ((4.0 / 3.0) * gj[0] * nx + gj[1] * ny);
                        M[1][i][j] -= aux * Ni * (gj[0] * nx + (4.0 / 3.0) * gj[1] * ny);
                        R[0][i] += aux * Ni * u[1][t[j]] * ((-2.0 / 3.0) * gj[1] * nx + gj[0] * ny);
                        R[1][i] += aux * Ni * u[0][t[j]] * (gj[1] * nx + (-2.0 / 3.0) * gj[0] * ny);
                    }
                }
            }
        }
        add_local(t, area[c], M[0], R[0], rowptr, col, val_x, rhs_x);
        add_local(t, area[c], M[1], R[1], rowptr, col, val_y, rhs_y);
    }
}

/* kIntegratePressureEquation :169-211 */
void or_assemble_pressure(int nc, const int* tri, const double* area, const double* invJ, const or_params* P,
                          const double* predx, const double* predy, const double* p_old,
                          const int* rowptr, const int* col, double* val, double* rhs)
{
    double qc[9], qw[3];
    const int nq = or_face_quadrature(1, qc, qw);
    for (int c = 0; c < nc; ++c) {
        const int* t = tri + 3 * c;
        const double* J = invJ + 4 * c;
        double M[3][3] = { { 0 } }, R[3] = { 0 };
        for (int q = 0; q < nq; ++q) {
            const double* L = qc + 3 * q;
            for (int i = 0; i < 3; ++i) {
                double gi[2];
                shape_grad(J, i, gi);
                const double aux = -P->rho / P->dt * L[i] * qw[q];
                for (int j = 0; j < 3; ++j) {
                    double gj[2];
                    shape_grad(J, j, gj);
                    const double vx = predx[t[j]], vy = predy[t[j]];
                    const double aux2 = (gi[0] * gj[0] + gi[1] * gj[1]) * qw[q];
                    M[i][j] += aux2;
                    if (p_old) R[i] += aux2 * p_old[t[j]];
                    R[i] += aux * (gj[0] * vx + gj[1] * vy);
                }
            }
        }
        add_local(t, area[c], M, R, rowptr, col, val, rhs);
    }
}

/* kIntegrateVelocityCorrection :213-259 */
void or_assemble_correction(int nc, const int* tri, const double* area, const double* invJ, const or_params* P,
                            const double* predx, const double* predy, const double* pres, const double* p_old,
                            const int* rowptr, const int* col, double* val_x, double* val_y,
                            double* rhs_x, double* rhs_y)
{
    double qc[9], qw[3];
    const int nq = or_face_quadrature(1, qc, qw);
    const double* pred[2] = { predx, predy };
    for (int c = 0; c < nc; ++c) {
        const int* t = tri + 3 * c;
        const double* J = invJ + 4 * c;
        double M[2][3][3] = { { { 0 } } }, R[2][3] = { { 0 } };
        for (int q = 0; q < nq; ++q) {
            const double* L = qc + 3 * q;
            for (int i = 0; i < 3; ++i) {
                const double Ni = L[i];
                const double aux2 = P->dt * Ni * qw[q];
                for (int j = 0; j < 3; ++j) {
                    double gj[2];
                    shape_grad(J, j, gj);
                    const double aux = P->rho * Ni * L[j] * qw[q];
                    double pv = pres[t[j]];
                    if (p_old) pv -= p_old[t[j]];
                    for (int k = 0; k < 2; ++k) {
                        M[k][i][j] += aux;
                        R[k][i] += aux * pred[k][t[j]] - aux2 * gj[k] * pv;
                    }
                }
            }
        }
        add_local(t, area[c], M[0], R[0], rowptr, col, val_x, rhs_x);
        add_local(t, area[c], M[1], R[1], rowptr, col, val_y, rhs_y);
    }
}

/* VelocityDirichletBCs::setDirichletValues :467-479 with kAccumulatePressureGradient
 * :261-289 and kFinalizePredictionBC :291-297: u*_bc = u_bc + dt/rho * sum(area grad_k
 * (p - p_old)) / sum(area) over the cells touching the boundary node. */
void or_prediction_bc(int nc, const int* tri, const double* area, const double* invJ, const or_params* P,
                      const double* pres, const double* p_old, int nbc, const int* bc_node,
                      const double* bc_val, const int* node_to_bc, int component, double* out_val)
{
    (void)bc_node;
    double* num = (double*)calloc(nbc > 0 ? nbc : 1, sizeof(double));
    double* den = (double*)calloc(nbc > 0 ? nbc : 1, sizeof(double));
    for (int c = 0; c < nc; ++c) {
        const int* t = tri + 3 * c;
        if (node_to_bc[t[0]] == -1 && node_to_bc[t[1]] == -1 && node_to_bc[t[2]] == -1) continue;
        const double* J = invJ + 4 * c;
        static const double sg[3][2] = { { 1.0, 0.0 }, { 0.0, 1.0 }, { -1.0, -1.0 } };
        double gx = 0.0, gy = 0.0;
        for (int i = 0; i < 3; ++i) {
            const double dp = pres[t[i]] - (p_old ? p_old[t[i]] : 0.0);
            gx += sg[i][0] * dp;
            gy += sg[i][1] * dp;
        }
        const double cgx = J[0] * gx + J[1] * gy;
        const double cgy = J[2] * gx + J[3] * gy;
        for (int i = 0; i < 3; ++i) {
            const int b = node_to_bc[t[i]];
            if (b != -1) {
                num[b] += area[c] * (component == 0 ? cgx : cgy);
                den[b] += area[c];
            }
        }
    }
    for (int b = 0; b < nbc; ++b) out_val[b] = bc_val[b] + P->dt / P->rho * num[b] / den[b];
    free(num);
    free(den);
}

/* boundaryLoadsCalculator :378-445 with kCountBodyEdges :299-320 and
 * kCalculateBodyForces :322-376 (first body edge of each cell, 2-point Gauss). */
int or_body_loads(int nc, const double* xy, const int* tri, const double* invJ, const int* edge_ids,
                  const or_params* P, const double* ux, const double* uy, const double* pres, double* cxcy)
{
    double ec[2], ew[2];
    const int ne = or_edge_quadrature(1, ec, ew);
    double F[4] = { 0, 0, 0, 0 };
    int nedges = 0;
    for (int c = 0; c < nc; ++c) {
        int e = -1;
        for (int i = 0; i < 3; ++i)
            if (edge_ids[3 * c + i] == P->body_id) { e = i; break; }
        if (e < 0) continue;
        ++nedges;
        const int* t = tri + 3 * c;
        const double* J = invJ + 4 * c;
        const int s = t[e], f = t[(e + 1) % 3];
        const double sx = xy[2 * s], sy = xy[2 * s + 1], fx = xy[2 * f], fy = xy[2 * f + 1];
        double nx = 0.5 * (sx + fx) - P->cx, ny = 0.5 * (sy + fy) - P->cy;
        const double inv = 1.0 / sqrt(nx * nx + ny * ny);
        nx *= inv; ny *= inv;
        const double half = 0.5 * sqrt((sx - fx) * (sx - fx) + (sy - fy) * (sy - fy));
        const double tx = ny, ty = -nx;
        double E[4] = { 0, 0, 0, 0 };
        for (int q = 0; q < ne; ++q) {
            const double qx = 0.5 * (ec[q] * (fx - sx) + (sx + fx));
            const double qy = 0.5 * (ec[q] * (fy - sy) + (sy + fy));
            const int v3 = t[2];
            const double dx = qx - xy[2 * v3], dy = qy - xy[2 * v3 + 1];
            double L[3];
            L[0] = J[0] * dx + J[2] * dy;
            L[1] = J[1] * dx + J[3] * dy;
            L[2] = 1.0 - L[0] - L[1];
            double pq = 0.0, dvt = 0.0;
            for (int i = 0; i < 3; ++i) {
                pq += pres[t[i]] * L[i];
                double g[2];
                shape_grad(J, i, g);
                dvt += (ux[t[i]] * tx + uy[t[i]] * ty) * (g[0] * nx + g[1] * ny);
            }
            const double w = ew[q] * half;
            E[0] -= pq * nx * w;
            E[1] -= pq * ny * w;
            E[2] += P->mu * dvt * tx * w;
            E[3] += P->mu * dvt * ty * w;
        }
        for (int k = 0; k < 4; ++k) F[k] += E[k];
    }
    const double coeff = 2.0 / (P->rho * P->mean_velocity * P->mean_velocity * P->thickness);
    cxcy[0] = (F[0] + F[2]) * coeff;
    cxcy[1] = (F[1] + F[3]) * coeff;
    return nedges;
}

/* ------------------------------------------------------------------------- */
/* One PFEM-2 time step, cases/Cylinder2D/main.cu:793-880. */
struct or_flow {
    or_params P;
    int nv, nc, nnz, np, cap;
    double* xy;
    int* tri;
    double *area, *invJ;
    int *nb_off, *nb_idx, *rowptr, *col, *edge_ids;
    double* centers;
    double* f[8]; /* ux, uy, ux_old, uy_old, pred_x, pred_y, p, p_old */
    double* A[5];
    double* b[5];
    int nbc[3];
    int* bc_node[3];
    double* bc_val[3];
    double* pred_bc_val[2];
    int* node_to_bc[2];
    double *px, *py, *l0, *l1, *l2, *pu, *pv;
    int* cell;
};

or_flow* or_flow_create(int nv, const double* xy, int nc, const int* tri, const or_params* p,
                        int nbu, const int* bu_node, const double* bu_val,
                        int nbv, const int* bv_node, const double* bv_val,
                        int nbp, const int* bp_node, const double* bp_val, int particle_cap)
{
    or_flow* f = (or_flow*)calloc(1, sizeof(or_flow));
    f->P = *p;
    f->nv = nv;
    f->nc = nc;
    f->xy = (double*)malloc(sizeof(double) * 2 * nv);
    memcpy(f->xy, xy, sizeof(double) * 2 * nv);
    f->tri = (int*)malloc(sizeof(int) * 3 * nc);
    memcpy(f->tri, tri, sizeof(int) * 3 * nc);
    f->area = (double*)malloc(sizeof(double) * nc);
    f->invJ = (double*)malloc(sizeof(double) * 4 * nc);
    or_mesh_geometry(nc, xy, tri, f->area, f->invJ);
    f->nb_off = (int*)malloc(sizeof(int) * (nc + 1));
    const int nnb = or_neighbors(nv, nc, tri, f->nb_off, NULL);
    f->nb_idx = (int*)malloc(sizeof(int) * (nnb > 0 ? nnb : 1));
    or_neighbors(nv, nc, tri, f->nb_off, f->nb_idx);
    f->rowptr = (int*)malloc(sizeof(int) * (nv + 1));
    f->nnz = or_csr_structure(nv, nc, tri, f->rowptr, NULL);
    f->col = (int*)malloc(sizeof(int) * f->nnz);
    or_csr_structure(nv, nc, tri, f->rowptr, f->col);
    f->edge_ids = (int*)malloc(sizeof(int) * 3 * nc);
    or_edge_boundary_ids(nc, xy, tri, p->lx, p->ly, p->has_cylinder, p->cx, p->cy, p->radius, f->edge_ids);
    for (int k = 0; k < 8; ++k) f->f[k] = (double*)calloc(nv, sizeof(double));
    for (int k = 0; k < 5; ++k) {
        f->A[k] = (double*)calloc(f->nnz, sizeof(double));
        f->b[k] = (double*)calloc(nv, sizeof(double));
    }
    const int nb[3] = { nbu, nbv, nbp };
    const int* bn[3] = { bu_node, bv_node, bp_node };
    const double* bv[3] = { bu_val, bv_val, bp_val };
    for (int k = 0; k < 3; ++k) {
        f->nbc[k] = nb[k];
        f->bc_node[k] = (int*)malloc(sizeof(int) * (nb[k] > 0 ? nb[k] : 1));
        f->bc_val[k] = (double*)malloc(sizeof(double) * (nb[k] > 0 ? nb[k] : 1));
        memcpy(f->bc_node[k], bn[k], sizeof(int) * nb[k]);
        memcpy(f->bc_val[k], bv[k], sizeof(double) * nb[k]);
    }
    for (int k = 0; k < 2; ++k) {
        f->pred_bc_val[k] = (double*)malloc(sizeof(double) * (nb[k] > 0 ? nb[k] : 1));
        f->node_to_bc[k] = (int*)malloc(sizeof(int) * nv);
        for (int i = 0; i < nv; ++i) f->node_to_bc[k][i] = -1;
        for (int b = 0; b < nb[k]; ++b) f->node_to_bc[k][bn[k][b]] = b;
    }
    f->centers = (double*)malloc(sizeof(double) * 3 * 16);
    const int lev = or_subcell_centers(p->level, f->centers);
    f->P.level = lev;
    const int np0 = nc * lev * lev;
    f->cap = particle_cap > np0 ? particle_cap : np0 * 2;
    double** arr[7] = { &f->px, &f->py, &f->l0, &f->l1, &f->l2, &f->pu, &f->pv };
    for (int k = 0; k < 7; ++k) *arr[k] = (double*)malloc(sizeof(double) * f->cap);
    f->cell = (int*)malloc(sizeof(int) * f->cap);
    f->np = or_seed(nc, xy, tri, lev, f->centers, f->px, f->py, f->l0, f->l1, f->l2, f->pu, f->pv, f->cell);
    /* initParticleVelocity from the (zero) initial velocity, Cylinder2D/main.cu:766 */
    or_correct_velocity(f->np, tri, f->cell, f->l0, f->l1, f->l2, f->f[0], f->f[1], NULL, NULL, f->pu, f->pv);
    return f;
}

void or_flow_destroy(or_flow* f)
{
    if (!f) return;
    free(f->xy); free(f->tri); free(f->area); free(f->invJ); free(f->nb_off); free(f->nb_idx);
    free(f->rowptr); free(f->col); free(f->edge_ids); free(f->centers);
    for (int k = 0; k < 8; ++k) free(f->f[k]);
    for (int k = 0; k < 5; ++k) { free(f->A[k]); free(f->b[k]); }
    for (int k = 0; k < 3; ++k) { free(f->bc_node[k]); free(f->bc_val[k]); }
    for (int k = 0; k < 2; ++k) { free(f->pred_bc_val[k]); free(f->node_to_bc[k]); }
    free(f->px); free(f->py); free(f->l0); free(f->l1); free(f->l2); free(f->pu); free(f->pv); free(f->cell);
    free(f);
}

int or_flow_step(or_flow* f, or_step_info* info)
{
    const or_params* P = &f->P;
    const int nv = f->nv, nnz = f->nnz;
    double *ux = f->f[0], *uy = f->f[1], *uxo = f->f[2], *uyo = f->f[3];
    double *prx = f->f[4], *pry = f->f[5], *pr = f->f[6], *pro = f->f[7];
    const double* pold = (P->scheme == 1) ? pro : NULL;
    int nd = 0, na = 0;
    const int nnew = or_advect(f->np, f->cap, f->px, f->py, f->l0, f->l1, f->l2, f->pu, f->pv, f->cell,
                               nv, f->xy, f->nc, f->tri, f->invJ, f->nb_off, f->nb_idx, ux, uy,
                               P->dt, P->substeps, P->level, f->centers, &nd, &na);
    if (nnew < 0) return -1;
    f->np = nnew;
    or_project(f->np, f->tri, f->cell, f->l0, f->l1, f->l2, f->pu, f->pv, nv, ux, uy);
    memcpy(uxo, ux, sizeof(double) * nv);
    memcpy(uyo, uy, sizeof(double) * nv);
    if (P->scheme == 1) memcpy(pro, pr, sizeof(double) * nv);
    int ok = 1;
    if (info) memset(info, 0, sizeof(*info));
    for (int it = 0; it < P->n_outer; ++it) {
        or_solve_info si;
        memset(f->A[0], 0, sizeof(double) * nnz); memset(f->A[1], 0, sizeof(double) * nnz);
        memset(f->b[0], 0, sizeof(double) * nv); memset(f->b[1], 0, sizeof(double) * nv);
        or_assemble_prediction(f->nc, f->xy, f->tri, f->area, f->invJ, f->edge_ids, P, ux, uy, uxo, uyo, pold,
                               f->rowptr, f->col, f->A[0], f->A[1], f->b[0], f->b[1]);
        for (int k = 0; k < 2; ++k) {
            or_prediction_bc(f->nc, f->tri, f->area, f->invJ, P, pr, pold, f->nbc[k], f->bc_node[k], f->bc_val[k],
                             f->node_to_bc[k], k, f->pred_bc_val[k]);
            or_apply_bcs(nv, f->rowptr, f->col, f->A[k], f->b[k], f->nbc[k], f->bc_node[k], f->pred_bc_val[k]);
            if (P->prediction_solver == 2)
                ok &= or_bicgstab(nv, f->rowptr, f->col, f->A[k], f->f[4 + k], f->b[k], P->tol, P->maxit,
                                  OR_PRECOND_JACOBI, 0, &si);
            else if (P->gmres_orth == 1)
                ok &= or_gmres_cgs2(nv, f->rowptr, f->col, f->A[k], f->f[4 + k], f->b[k], P->tol, P->maxit,
                                    OR_PRECOND_JACOBI, &si);
            else
                ok &= or_gmres(nv, f->rowptr, f->col, f->A[k], f->f[4 + k], f->b[k], P->tol, P->maxit,
                               OR_PRECOND_JACOBI, &si);
            if (info && it < 8) info->it_pred[k][it] = si.iterations;
        }
        memset(f->A[2], 0, sizeof(double) * nnz);
        memset(f->b[2], 0, sizeof(double) * nv);
        or_assemble_pressure(f->nc, f->tri, f->area, f->invJ, P, prx, pry, pold, f->rowptr, f->col, f->A[2], f->b[2]);
        or_apply_bcs(nv, f->rowptr, f->col, f->A[2], f->b[2], f->nbc[2], f->bc_node[2], f->bc_val[2]);
        double relres = 0.0;
        const double ptol = P->pressure_tol > 0 ? P->pressure_tol : P->tol;
        const int pmaxit = P->pressure_maxit > 0 ? P->pressure_maxit : P->maxit;
        if (P->pressure_ordering == 0 && P->pressure_criterion == 0)
            ok &= or_pcg(nv, f->rowptr, f->col, f->A[2], pr, f->b[2], ptol, pmaxit, P->pressure_precond, &si);
        else
            ok &= or_cg(nv, f->rowptr, f->col, f->A[2], pr, f->b[2], ptol, pmaxit, P->pressure_precond,
                        P->pressure_ordering, P->pressure_criterion, &si, &relres);
        if (info && it < 8) {
            info->it_pres[it] = si.iterations;
            info->res_pres[it] = relres;
        }
        memset(f->A[3], 0, sizeof(double) * nnz); memset(f->A[4], 0, sizeof(double) * nnz);
        memset(f->b[3], 0, sizeof(double) * nv); memset(f->b[4], 0, sizeof(double) * nv);
        or_assemble_correction(f->nc, f->tri, f->area, f->invJ, P, prx, pry, pr, pold, f->rowptr, f->col,
                               f->A[3], f->A[4], f->b[3], f->b[4]);
        for (int k = 0; k < 2; ++k) {
            or_apply_bcs(nv, f->rowptr, f->col, f->A[3 + k], f->b[3 + k], f->nbc[k], f->bc_node[k], f->bc_val[k]);
            ok &= or_pcg(nv, f->rowptr, f->col, f->A[3 + k], f->f[k], f->b[3 + k], P->tol, P->maxit,
                         OR_PRECOND_JACOBI, &si);
            if (info && it < 8) info->it_corr[k][it] = si.iterations;
        }
    }
    or_correct_velocity(f->np, f->tri, f->cell, f->l0, f->l1, f->l2, ux, uy, uxo, uyo, f->pu, f->pv);
    if (info) {
        info->particles = f->np;
        info->deleted = nd;
        info->added = na;
        info->conv_ok = ok;
        if (P->calc_loads) {
            double cc[2];
            or_body_loads(f->nc, f->xy, f->tri, f->invJ, f->edge_ids, P, ux, uy, pr, cc);
            info->cx = cc[0];
            info->cy = cc[1];
        }
    }
    return 0;
}

int or_flow_particle_count(const or_flow* f) { return f->np; }

void or_flow_set_solvers(or_flow* f, int pressure_precond, int pressure_ordering, int prediction_solver,
                         int gmres_orth, int pressure_criterion)
{
    f->P.pressure_precond = pressure_precond;
    f->P.pressure_ordering = pressure_ordering;
    f->P.prediction_solver = prediction_solver;
    f->P.gmres_orth = gmres_orth;
    f->P.pressure_criterion = pressure_criterion;
}

void or_flow_get_field(const or_flow* f, int which, double* out) { memcpy(out, f->f[which], sizeof(double) * f->nv); }
void or_flow_set_field(or_flow* f, int which, const double* in) { memcpy(f->f[which], in, sizeof(double) * f->nv); }

void or_flow_get_particles(const or_flow* f, double* px, double* py, double* l0, double* l1, double* l2,
                           double* pu, double* pv, int* cell)
{
    const size_t n = sizeof(double) * f->np;
    memcpy(px, f->px, n); memcpy(py, f->py, n); memcpy(l0, f->l0, n); memcpy(l1, f->l1, n);
    memcpy(l2, f->l2, n); memcpy(pu, f->pu, n); memcpy(pv, f->pv, n);
    memcpy(cell, f->cell, sizeof(int) * f->np);
}

void or_flow_set_particles(or_flow* f, int np, const double* px, const double* py, const double* l0,
                           const double* l1, const double* l2, const double* pu, const double* pv, const int* cell)
{
    if (np > f->cap) return;
    const size_t n = sizeof(double) * np;
    f->np = np;
    memcpy(f->px, px, n); memcpy(f->py, py, n); memcpy(f->l0, l0, n); memcpy(f->l1, l1, n);
    memcpy(f->l2, l2, n); memcpy(f->pu, pu, n); memcpy(f->pv, pv, n);
    memcpy(f->cell, cell, sizeof(int) * np);
}

int or_flow_csr_nnz(const or_flow* f) { return f->nnz; }

void or_flow_get_matrix(const or_flow* f, int which, double* val, double* rhs)
{
    if (val) memcpy(val, f->A[which], sizeof(double) * f->nnz);
    if (rhs) memcpy(rhs, f->b[which], sizeof(double) * f->nv);
}

/* ------------------------------------------------------------------------- */
/* Learned initial guess: the network of pf2_oracle.h (no reference counterpart). */
#define MH OR_MPNN_H
int or_mpnn_param_count(void) { return MH * OR_MPNN_IN + MH + OR_MPNN_LAYERS * (MH * 2 * MH + MH) + MH + 1; }

typedef struct {
    const double *W0, *c0, *W[OR_MPNN_LAYERS], *c[OR_MPNN_LAYERS], *w4, *c4;
} mpnn_view;

static mpnn_view mpnn_split(const double* th)
{
    mpnn_view v;
    v.W0 = th; th += MH * OR_MPNN_IN;
    v.c0 = th; th += MH;
    for (int l = 0; l < OR_MPNN_LAYERS; ++l) { v.W[l] = th; th += MH * 2 * MH; v.c[l] = th; th += MH; }
    v.w4 = th; th += MH;
    v.c4 = th;
    return v;
}

/* h[(l+1)][n][MH] for l = 0..LAYERS (h[0] after the encoder), m[l][n][MH], z0 and z[l] kept */
typedef struct { double *h, *m, *z; } mpnn_acts;

static void mpnn_fwd(int n, const int* rp, const int* col, const double* f, mpnn_view P, mpnn_acts* A, double* y)
{
    const int L = OR_MPNN_LAYERS;
    double* h0 = A->h;
    for (int i = 0; i < n; ++i)
        for (int o = 0; o < MH; ++o) {
            double s = P.c0[o];
            for (int k = 0; k < OR_MPNN_IN; ++k) s += P.W0[o * OR_MPNN_IN + k] * f[i * OR_MPNN_IN + k];
            A->z[i * MH + o] = s;
            h0[i * MH + o] = s > 0 ? s : 0;
        }
    for (int l = 0; l < L; ++l) {
        const double* hp = A->h + (size_t)l * n * MH;
        double* hn = A->h + (size_t)(l + 1) * n * MH;
        double* m = A->m + (size_t)l * n * MH;
        double* z = A->z + (size_t)(l + 1) * n * MH;
        for (int i = 0; i < n; ++i) {
            int d = 0;
            for (int o = 0; o < MH; ++o) m[i * MH + o] = 0;
            for (int k = rp[i]; k < rp[i + 1]; ++k) {
                if (col[k] == i) continue;
                ++d;
                for (int o = 0; o < MH; ++o) m[i * MH + o] += hp[col[k] * MH + o];
            }
            for (int o = 0; o < MH; ++o) m[i * MH + o] = d ? m[i * MH + o] / d : 0.0;
        }
        for (int i = 0; i < n; ++i)
            for (int o = 0; o < MH; ++o) {
                double s = P.c[l][o];
                const double* w = P.W[l] + o * 2 * MH;
                for (int k = 0; k < MH; ++k) s += w[k] * hp[i * MH + k] + w[MH + k] * m[i * MH + k];
                z[i * MH + o] = s;
                hn[i * MH + o] = hp[i * MH + o] + (s > 0 ? s : 0);
            }
    }
    const double* hl = A->h + (size_t)L * n * MH;
    for (int i = 0; i < n; ++i) {
        double s = P.c4[0];
        for (int o = 0; o < MH; ++o) s += P.w4[o] * hl[i * MH + o];
        y[i] = s;
    }
}

static mpnn_acts mpnn_alloc(int n)
{
    mpnn_acts A;
    A.h = (double*)calloc((size_t)(OR_MPNN_LAYERS + 1) * n * MH, sizeof(double));
    A.m = (double*)calloc((size_t)OR_MPNN_LAYERS * n * MH, sizeof(double));
    A.z = (double*)calloc((size_t)(OR_MPNN_LAYERS + 1) * n * MH, sizeof(double));
    return A;
}

static void mpnn_free(mpnn_acts* A) { free(A->h); free(A->m); free(A->z); }

double or_mpnn_forward(int n, const int* rp, const int* col, const double* f, const double* th, double* y,
                       const double* t)
{
    mpnn_acts A = mpnn_alloc(n);
    mpnn_fwd(n, rp, col, f, mpnn_split(th), &A, y);
    mpnn_free(&A);
    double loss = 0.0;
    if (t) {
        for (int i = 0; i < n; ++i) loss += (y[i] - t[i]) * (y[i] - t[i]);
        loss /= n;
    }
    return loss;
}

double or_mpnn_backward(int n, const int* rp, const int* col, const double* f, const double* th, const double* t,
                        double* grad)
{
    const int L = OR_MPNN_LAYERS;
    const mpnn_view P = mpnn_split(th);
    memset(grad, 0, sizeof(double) * or_mpnn_param_count());
    double* gW0 = grad;
    double* gc0 = gW0 + MH * OR_MPNN_IN;
    double* gW[OR_MPNN_LAYERS];
    double* gc[OR_MPNN_LAYERS];
    double* g = gc0 + MH;
    for (int l = 0; l < L; ++l) { gW[l] = g; g += MH * 2 * MH; gc[l] = g; g += MH; }
    double* gw4 = g;
    double* gc4 = g + MH;
    mpnn_acts A = mpnn_alloc(n);
    double* y = (double*)malloc(sizeof(double) * n);
    mpnn_fwd(n, rp, col, f, P, &A, y);
    double loss = 0.0;
    double* dh = (double*)calloc((size_t)n * MH, sizeof(double));
    double* dm = (double*)calloc((size_t)n * MH, sizeof(double));
    const double* hl = A.h + (size_t)L * n * MH;
    for (int i = 0; i < n; ++i) {
        const double r = y[i] - t[i];
        loss += r * r;
        const double dy = 2.0 * r / n;
        gc4[0] += dy;
        for (int o = 0; o < MH; ++o) { gw4[o] += dy * hl[i * MH + o]; dh[i * MH + o] = dy * P.w4[o]; }
    }
    for (int l = L - 1; l >= 0; --l) {
        const double* hp = A.h + (size_t)l * n * MH;
        const double* m = A.m + (size_t)l * n * MH;
        const double* z = A.z + (size_t)(l + 1) * n * MH;
        for (int i = 0; i < n; ++i)
            for (int o = 0; o < MH; ++o) dm[i * MH + o] = 0.0;
        /* dz = dh * [z > 0]; dW += dz [h; m]^T; [dh_self; dm] = W^T dz; dh (residual) stays */
        double* dself = (double*)calloc((size_t)n * MH, sizeof(double));
        for (int i = 0; i < n; ++i)
            for (int o = 0; o < MH; ++o) {
                const double dz = z[i * MH + o] > 0 ? dh[i * MH + o] : 0.0;
                if (dz == 0.0) continue;
                gc[l][o] += dz;
                double* gw = gW[l] + o * 2 * MH;
                const double* w = P.W[l] + o * 2 * MH;
                for (int k = 0; k < MH; ++k) {
                    gw[k] += dz * hp[i * MH + k];
                    gw[MH + k] += dz * m[i * MH + k];
                    dself[i * MH + k] += w[k] * dz;
                    dm[i * MH + k] += w[MH + k] * dz;
                }
            }
        /* m_i = mean_j h_j: h_j receives dm_i / d_i from each neighbour i */
        for (int i = 0; i < n; ++i) {
            int d = 0;
            for (int k = rp[i]; k < rp[i + 1]; ++k) d += (col[k] != i);
            if (!d) continue;
            for (int k = rp[i]; k < rp[i + 1]; ++k) {
                if (col[k] == i) continue;
                for (int o = 0; o < MH; ++o) dself[col[k] * MH + o] += dm[i * MH + o] / d;
            }
        }
        for (size_t q = 0; q < (size_t)n * MH; ++q) dh[q] += dself[q];
        free(dself);
    }
    for (int i = 0; i < n; ++i)
        for (int o = 0; o < MH; ++o) {
            const double dz = A.z[i * MH + o] > 0 ? dh[i * MH + o] : 0.0;
            gc0[o] += dz;
            for (int k = 0; k < OR_MPNN_IN; ++k) gW0[o * OR_MPNN_IN + k] += dz * f[i * OR_MPNN_IN + k];
        }
    free(dh); free(dm); free(y);
    mpnn_free(&A);
    return loss / n;
}

/* AdamW (decoupled weight decay), bias-corrected; `step` counts from 1. */
void or_adamw(int np, double* th, const double* g, double* m, double* v, int step, double lr, double b1, double b2,
              double eps, double wd)
{
    const double c1 = 1.0 - pow(b1, step), c2 = 1.0 - pow(b2, step);
    for (int k = 0; k < np; ++k) {
        m[k] = b1 * m[k] + (1.0 - b1) * g[k];
        v[k] = b2 * v[k] + (1.0 - b2) * g[k] * g[k];
        th[k] -= lr * (m[k] / c1 / (sqrt(v[k] / c2) + eps) + wd * th[k]);
    }
}
