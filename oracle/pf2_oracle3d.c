/* pf2_oracle3d.c - CPU restatement of the reference's 3D path (TEST INFRASTRUCTURE
 * ONLY: the parity tests and nothing else call it).
 *
 * Mesh3D geometry and neighbour lists (src/mesh_3d.cu:12-35, :158-196), the node-graph
 * CSR pattern (src/linear_algebra/sparse_matrix.cu:56-97) and the Poisson3D assembly
 * (cases/Poisson3D/main.cu:22-67 with addLocalToGlobal3D,
 * src/integration/numerical_integrator_3d.cuh:25-46), single-threaded FP64 in the
 * reference's element order.  The reference sums with atomics, so its matrix is only
 * reproducible to rounding; this oracle fixes the order (cells ascending). */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "pf2_oracle.h"

static int cmp_int3(const void* a, const void* b)
{
    const int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}

/* kCalculateCellVolume, kCalculateInvJacobi (mesh_3d.cu:12-35) with
 * GenericMatrix3x3::det / inverse (src/common/matrix3x3.cuh): rows e_k = v_k - v_3,
 * volume = |e_0 . (e_1 x e_2)| / 6, invJ = adj(J) / det J, zero when |det J| < 2e-6. */
void or_mesh3d_geometry(int nc, const double* xyz, const int* tet, double* volume, double* invJ)
{
    for (int c = 0; c < nc; ++c) {
        const double* p[4];
        for (int k = 0; k < 4; ++k) p[k] = xyz + 3 * tet[4 * c + k];
        double d[9];
        for (int r = 0; r < 3; ++r)
            for (int k = 0; k < 3; ++k) d[3 * r + k] = p[r][k] - p[3][k];
        /* cross(e1, e2) then e0 . it */
        const double cx = d[4] * d[8] - d[5] * d[7];
        const double cy = d[5] * d[6] - d[3] * d[8];
        const double cz = d[3] * d[7] - d[4] * d[6];
        volume[c] = fabs(d[0] * cx + d[1] * cy + d[2] * cz) * (1.0 / 6.0);
        const double det = d[0] * (d[4] * d[8] - d[5] * d[7]) - d[1] * (d[3] * d[8] - d[5] * d[6]) +
                           d[2] * (d[3] * d[7] - d[4] * d[6]);
        double* J = invJ + 9 * c;
        if (fabs(det) < 2e-6) {
            for (int k = 0; k < 9; ++k) J[k] = 0.0;
            continue;
        }
        const double r = 1.0 / det;
        J[0] = r * (d[4] * d[8] - d[5] * d[7]);
        J[1] = r * (d[2] * d[7] - d[1] * d[8]);
        J[2] = r * (d[1] * d[5] - d[2] * d[4]);
        J[3] = r * (d[5] * d[6] - d[3] * d[8]);
        J[4] = r * (d[0] * d[8] - d[2] * d[6]);
        J[5] = r * (d[2] * d[3] - d[0] * d[5]);
        J[6] = r * (d[3] * d[7] - d[4] * d[6]);
        J[7] = r * (d[1] * d[6] - d[0] * d[7]);
        J[8] = r * (d[0] * d[4] - d[1] * d[3]);
    }
}

/* Mesh3D::fillCellNeighborIndicesCPU (mesh_3d.cu:158-196): all pairs i < j, neighbours
 * when they share three vertices, each list ascending.  O(nc^2): small meshes only.
 * idx may be NULL (count only); returns the number of entries. */
int or_mesh3d_neighbors(int nc, const int* tet, int* offsets, int* idx)
{
    int* cnt = (int*)calloc((size_t)nc + 1, sizeof(int));
    int* first = NULL;
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1) {
            offsets[0] = 0;
            for (int i = 0; i < nc; ++i) offsets[i + 1] = offsets[i] + cnt[i];
            if (!idx) break;
            first = (int*)malloc(sizeof(int) * ((size_t)nc + 1));
            memcpy(first, offsets, sizeof(int) * ((size_t)nc + 1));
        }
        for (int i = 0; i < nc; ++i)
            for (int j = i + 1; j < nc; ++j) {
                int common = 0;
                for (int a = 0; a < 4; ++a)
                    for (int b = 0; b < 4; ++b)
                        if (tet[4 * i + a] == tet[4 * j + b]) {
                            ++common;
                            break;
                        }
                if (common != 3) continue;
                if (pass == 0) {
                    ++cnt[i];
                    ++cnt[j];
                } else {
                    idx[first[i]++] = j;
                    idx[first[j]++] = i;
                }
            }
    }
    /* the pairs arrive with i ascending for j's list and j ascending for i's: sort */
    if (idx)
        for (int i = 0; i < nc; ++i) qsort(idx + offsets[i], (size_t)(offsets[i + 1] - offsets[i]), sizeof(int), cmp_int3);
    const int total = offsets[nc];
    free(cnt);
    free(first);
    return total;
}

/* SparseMatrixCSR::initialize(const Mesh3D&) (sparse_matrix.cu:56-97): row i holds
 * {i} U the vertices of every tetrahedron containing i, ascending.  col may be NULL. */
int or_csr_structure_3d(int nv, int nc, const int* tet, int* rowptr, int* col)
{
    int* deg = (int*)calloc((size_t)nv + 1, sizeof(int));
    for (int c = 0; c < 4 * nc; ++c) ++deg[tet[c]];
    int* off = (int*)malloc(sizeof(int) * ((size_t)nv + 1));
    off[0] = 0;
    for (int i = 0; i < nv; ++i) off[i + 1] = off[i] + deg[i];
    int* cells = (int*)malloc(sizeof(int) * ((size_t)off[nv] + 1));
    int* fill = (int*)calloc((size_t)nv + 1, sizeof(int));
    for (int c = 0; c < nc; ++c)
        for (int k = 0; k < 4; ++k) {
            const int v = tet[4 * c + k];
            cells[off[v] + fill[v]++] = c;
        }
    int total = 0;
    rowptr[0] = 0;
    int* buf = (int*)malloc(sizeof(int) * (1 + 4 * 1024));
    for (int i = 0; i < nv; ++i) {
        int m = 0;
        buf[m++] = i;
        for (int q = off[i]; q < off[i + 1] && m + 4 <= 1 + 4 * 1024; ++q)
            for (int k = 0; k < 4; ++k) buf[m++] = tet[4 * cells[q] + k];
        qsort(buf, (size_t)m, sizeof(int), cmp_int3);
        int u = 0;
        for (int q = 0; q < m; ++q)
            if (q == 0 || buf[q] != buf[q - 1]) {
                if (col) col[total + u] = buf[q];
                ++u;
            }
        total += u;
        rowptr[i + 1] = total;
    }
    free(buf);
    free(fill);
    free(cells);
    free(off);
    free(deg);
    return total;
}

/* createCellQuadratureFormula(1) (src/integration/quadrature_formula_3d.cu, case 1):
 * coords4 gets (x, y, z, 1 - x - y - z) per point; returns the number of points. */
int or_cell_quadrature_3d(double* coords4, double* weights)
{
    static const double xyz[6][3] = { { 0.0701026973651683, 0.166660699730426, 0.596575741463645 },
                                      { 0.168695371477743, 0.584652626698847, 0.168695218708539 },
                                      { 0.418175789241166, 0.0803037256707293, 0.418101348156118 },
                                      { 0.596576288848820, 0.166672635105983, 0.0700786026978242 },
                                      { 0.164808547352848, 0.0851134715186107, 0.164808684755350 },
                                      { 0.0731475667668616, 0.440339136918213, 0.0731570614497775 } };
    static const double w[6] = { 0.180396407632724, 0.193316294293662, 0.133594798870359,
                                 0.180371079146698, 0.201016720944591, 0.111304699111967 };
    for (int k = 0; k < 6; ++k) {
        coords4[4 * k] = xyz[k][0];
        coords4[4 * k + 1] = xyz[k][1];
        coords4[4 * k + 2] = xyz[k][2];
        coords4[4 * k + 3] = ((1.0 - xyz[k][0]) - xyz[k][1]) - xyz[k][2];
        weights[k] = w[k];
    }
    return 6;
}

static double rhs3d(int kind, double x, double y, double z)
{
    if (kind == 0) return exp(-(x * x + 10 * y * y + z * z)); /* Poisson3D/main.cu:22-24 */
    const double pi = 3.14159265358979323846;
    return 3.0 * pi * pi * sin(pi * x) * sin(pi * y) * sin(pi * z);
}

/* kIntegrateOverCell (Poisson3D/main.cu:26-67) + addLocalToGlobal3D: per cell, with
 * G_j = invJ * grad N_j (shapeFuncGrad3D: e_0, e_1, e_2, (-1,-1,-1)), local (i, j) +=
 * lambda (G_i . G_j) w_q and rhs_i += f(x_q) L_i(q) w_q over the points, then scatter
 * local * volume. */
void or_assemble_poisson_3d(int nc, const double* xyz, const int* tet, const double* volume, const double* invJ,
                            int rhs_kind, double lambda, const int* rowptr, const int* col, double* val,
                            double* rhs)
{
    double L[24], w[6];
    const int nq = or_cell_quadrature_3d(L, w);
    for (int c = 0; c < nc; ++c) {
        const int* t = tet + 4 * c;
        const double* J = invJ + 9 * c;
        double G[4][3];
        for (int r = 0; r < 3; ++r) {
            G[0][r] = J[3 * r];
            G[1][r] = J[3 * r + 1];
            G[2][r] = J[3 * r + 2];
            G[3][r] = -((G[0][r] + G[1][r]) + G[2][r]);
        }
        double M[4][4] = { { 0 } }, R[4] = { 0 };
        for (int q = 0; q < nq; ++q) {
            const double* l = L + 4 * q;
            double X[3];
            for (int a = 0; a < 3; ++a)
                X[a] = l[0] * xyz[3 * t[0] + a] + l[1] * xyz[3 * t[1] + a] + l[2] * xyz[3 * t[2] + a] +
                       l[3] * xyz[3 * t[3] + a];
            const double f = rhs3d(rhs_kind, X[0], X[1], X[2]);
            for (int i = 0; i < 4; ++i) {
                for (int j = 0; j < 4; ++j) {
                    const double d = G[i][0] * G[j][0] + G[i][1] * G[j][1] + G[i][2] * G[j][2];
                    M[i][j] += lambda * d * w[q];
                }
                R[i] += f * l[i] * w[q];
            }
        }
        for (int i = 0; i < 4; ++i) {
            for (int j = 0; j < 4; ++j) {
                const int k = or_find_in_row(rowptr, col, t[i], t[j]);
                if (k >= 0) val[k] += M[i][j] * volume[c];
            }
            rhs[t[i]] += R[i] * volume[c];
        }
    }
}
