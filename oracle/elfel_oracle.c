/*
 * CPU oracle for the Elfel.jl element-integration / assembly / solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark call it; the
 * GPU library never links it.
 *
 * It restates, in plain C, the algorithm of the reference (Elfel.jl v0.4.0):
 *   - basis functions and parametric gradients of T3/T6
 *       src/FElements.jl:239-246 (T3), :264-288 (T6)
 *   - Jacobian matrix J = sum_j x_j (x) gradNpar_j and det J
 *       src/FElements.jl:148-168 (_jac, jacjac), :120-129 (Jacobian Val{2})
 *   - spatial gradients gradN = gradNpar / J
 *       src/QPIterators.jl:132-140 (bfungrad)
 *   - the user weak forms integrated per element
 *       heat        test/test_heat.jl:41-58
 *       elasticity  test/test_elasticity.jl:150-171
 *       Stokes TH   test/test_stokes.jl:629-657 (vector Laplacian form)
 *                   test/test_stokes.jl:364-400 (Reddy form, scalar spaces)
 *   - local matrix layout: init! fills row/col column-major
 *       src/LocalAssemblers.jl:68-83
 *   - COO -> CSC with duplicates summed in input order, zeros kept
 *       src/Assemblers.jl:121-123 -> SparseArrays.sparse (Julia stdlib)
 *   - a Jacobi-preconditioned CG in FP64 (the CPU baseline of the solve;
 *       the reference itself calls a direct solver, test/test_heat.jl:73-76)
 *
 * All index arrays are 0-based here; the Python wrapper converts.
 * Compile: gcc -O2 -fPIC -shared -ffp-contract=off -fopenmp
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------- basis functions (src/FElements.jl) ---------------- */

static void bfun_t3(double r, double s, double* N) {
    N[0] = 1.0 - r - s;
    N[1] = r;
    N[2] = s;
}
static void gradpar_t3(double r, double s, double* G /* 3x2 */) {
    (void)r; (void)s;
    G[0] = -1.0; G[1] = -1.0;
    G[2] = 1.0;  G[3] = 0.0;
    G[4] = 0.0;  G[5] = 1.0;
}
static void bfun_t6(double r, double s, double* N) {
    double t = 1.0 - r - s;
    N[0] = t * (t + t - 1);
    N[1] = r * (r + r - 1);
    N[2] = s * (s + s - 1);
    N[3] = 4 * r * t;
    N[4] = 4 * r * s;
    N[5] = 4 * s * t;
}
static void gradpar_t6(double r, double s, double* G /* 6x2 */) {
    G[0] = -3 + 4 * r + 4 * s;  G[1] = -3 + 4 * r + 4 * s;
    G[2] = 4 * r - 1;           G[3] = 0.0;
    G[4] = 0.0;                 G[5] = 4 * s - 1;
    G[6] = 4 - 8 * r - 4 * s;   G[7] = -4 * r;
    G[8] = 4 * s;               G[9] = 4 * r;
    G[10] = -4 * s;             G[11] = 4 - 4 * r - 8 * s;
}

/* Fill N (npts x nn) and G (npts x nn x 2) tables for element with nn nodes
 * (3 or 6) at the given quadrature points (QPIterators.jl:14-50). */
int oracle_bfun_tables(int nn, int npts, const double* pc, double* N, double* G) {
    for (int q = 0; q < npts; ++q) {
        double r = pc[2 * q], s = pc[2 * q + 1];
        if (nn == 3) { bfun_t3(r, s, N + 3 * q); gradpar_t3(r, s, G + 6 * q); }
        else if (nn == 6) { bfun_t6(r, s, N + 6 * q); gradpar_t6(r, s, G + 12 * q); }
        else return -1;
    }
    return 0;
}

/* J[a][b] = sum_j x_j[a] * Gpar_j[b]  (FElements.jl:148-156), det (:120-129),
 * gradN_j = Gpar_j * inv(J)  (QPIterators.jl:132-140). Returns det. */
static double jac_and_grad(int nn, const int64_t* conn, const double* xy, const double* Gq,
                           double* gN /* nn x 2 */) {
    double J11 = 0, J12 = 0, J21 = 0, J22 = 0;
    for (int j = 0; j < nn; ++j) {
        const double x = xy[2 * conn[j]], y = xy[2 * conn[j] + 1];
        J11 += x * Gq[2 * j];
        J12 += x * Gq[2 * j + 1];
        J21 += y * Gq[2 * j];
        J22 += y * Gq[2 * j + 1];
    }
    double det = J11 * J22 - J21 * J12;
    /* row vector g times inv(J): inv(J) = [J22 -J12; -J21 J11] / det */
    for (int j = 0; j < nn; ++j) {
        double g1 = Gq[2 * j], g2 = Gq[2 * j + 1];
        gN[2 * j] = (g1 * J22 - g2 * J21) / det;
        gN[2 * j + 1] = (-g1 * J12 + g2 * J11) / det;
    }
    return det;
}

/*
 * Heat conduction element matrices and load vectors (test/test_heat.jl:41-58):
 *   ke[i,j] += dot(gradN_i, gradN_j) * (kappa_e * JxW),   fe[j] += N_j * Q * JxW
 * ke is stored per element column-major (entry (i,j) at i + j*nn), the order in
 * which LocalMatrixAssembler.init! lists its row/col numbers.
 */
void oracle_heat(int nn, int npts, const double* N, const double* G, const double* w,
                 int64_t nel, const int64_t* conn, const double* xy,
                 const double* kappa, double Q, double* ke, double* fe) {
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < nel; ++e) {
        const int64_t* c = conn + e * nn;
        double* k = ke + e * nn * nn;
        double* f = fe + e * nn;
        double gN[12];
        for (int i = 0; i < nn * nn; ++i) k[i] = 0.0;
        for (int i = 0; i < nn; ++i) f[i] = 0.0;
        for (int q = 0; q < npts; ++q) {
            double det = jac_and_grad(nn, c, xy, G + q * nn * 2, gN);
            double JxW = det * w[q];
            const double* Nq = N + q * nn;
            for (int j = 0; j < nn; ++j) {
                for (int i = 0; i < nn; ++i)
                    k[i + j * nn] += (gN[2 * i] * gN[2 * j] + gN[2 * i + 1] * gN[2 * j + 1]) * (kappa[e] * JxW);
                f[j] += Nq[j] * Q * JxW;
            }
        }
    }
}

/*
 * Linear elasticity, vector space with 2 components (test/test_elasticity.jl:150-171).
 * DOFs node-major, component-minor: dof k -> node k/2, component k%2.
 * B(g,1) = (g1, 0, g2), B(g,2) = (0, g2, g1); ke[i,j] += dot(D*B_j, B_i) * JxW.
 * Body force b_e (2 per element, constant): fe[k] += N_node * b_e[comp] * JxW.
 */
void oracle_elasticity(int nn, int npts, const double* N, const double* G, const double* w,
                       int64_t nel, const int64_t* conn, const double* xy, const double* D /* 3x3 row-major */,
                       const double* bforce /* nel x 2 or NULL */, double* ke, double* fe) {
    const int nd = 2 * nn;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < nel; ++e) {
        const int64_t* c = conn + e * nn;
        double* k = ke + e * nd * nd;
        double* f = fe + e * nd;
        double gN[12];
        for (int i = 0; i < nd * nd; ++i) k[i] = 0.0;
        for (int i = 0; i < nd; ++i) f[i] = 0.0;
        for (int q = 0; q < npts; ++q) {
            double det = jac_and_grad(nn, c, xy, G + q * nn * 2, gN);
            double JxW = det * w[q];
            for (int j = 0; j < nd; ++j) {
                int nj = j / 2, cj = j % 2;
                double Bj[3];
                if (cj == 0) { Bj[0] = gN[2 * nj]; Bj[1] = 0; Bj[2] = gN[2 * nj + 1]; }
                else { Bj[0] = 0; Bj[1] = gN[2 * nj + 1]; Bj[2] = gN[2 * nj]; }
                double DBj[3];
                for (int a = 0; a < 3; ++a) DBj[a] = D[3 * a] * Bj[0] + D[3 * a + 1] * Bj[1] + D[3 * a + 2] * Bj[2];
                for (int i = 0; i < nd; ++i) {
                    int ni = i / 2, ci = i % 2;
                    double Bi[3];
                    if (ci == 0) { Bi[0] = gN[2 * ni]; Bi[1] = 0; Bi[2] = gN[2 * ni + 1]; }
                    else { Bi[0] = 0; Bi[1] = gN[2 * ni + 1]; Bi[2] = gN[2 * ni]; }
                    k[i + j * nd] += (DBj[0] * Bi[0] + DBj[1] * Bi[1] + DBj[2] * Bi[2]) * JxW;
                }
            }
            if (bforce) {
                const double* Nq = N + q * nn;
                for (int j = 0; j < nd; ++j) f[j] += Nq[j / 2] * bforce[2 * e + (j % 2)] * JxW;
            }
        }
    }
}

/*
 * Taylor-Hood Stokes, vector-Laplacian form (test/test_stokes.jl:629-657):
 * velocity vector T6 (12 dofs, node-major/component-minor), pressure T3 (3 dofs).
 * The Jacobian comes from the velocity element.
 *   kuu[i,j] += (mu*JxW) * dot(gradNu_i, gradNu_j)  if comp(i) == comp(j), else stays 0
 *   kup[i,j] += (-JxW * Np_j) * gradNu_i[comp(i)]
 * kuu 12x12 and kup 12x3 are column-major per element.
 * Np (npts x 3) is the pressure basis at the same quadrature points.
 */
void oracle_stokes_veclap(int npts, const double* Nu, const double* Gu, const double* Np, const double* w,
                          int64_t nel, const int64_t* uconn, const double* xy, double mu,
                          double* kuu, double* kup) {
    (void)Nu;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < nel; ++e) {
        const int64_t* c = uconn + e * 6;
        double* ku = kuu + e * 144;
        double* kp = kup + e * 36;
        double gN[12];
        for (int i = 0; i < 144; ++i) ku[i] = 0.0;
        for (int i = 0; i < 36; ++i) kp[i] = 0.0;
        for (int q = 0; q < npts; ++q) {
            double det = jac_and_grad(6, c, xy, Gu + q * 12, gN);
            double JxW = det * w[q];
            for (int j = 0; j < 12; ++j)
                for (int i = 0; i < 12; ++i)
                    if ((i % 2) == (j % 2)) {
                        int a = i / 2, b = j / 2;
                        ku[i + 12 * j] += (mu * JxW) * (gN[2 * a] * gN[2 * b] + gN[2 * a + 1] * gN[2 * b + 1]);
                    }
            for (int j = 0; j < 3; ++j)
                for (int i = 0; i < 12; ++i)
                    kp[i + 12 * j] += (-JxW * Np[3 * q + j]) * gN[2 * (i / 2) + (i % 2)];
        }
    }
}

/*
 * Taylor-Hood Stokes, "Reddy" form with scalar velocity spaces
 * (test/test_stokes.jl:364-400).  Jacobian from the pressure (T3) element.
 * Blocks per element, column-major: kxx 6x6, kyy 6x6, kxy 6x6, kxp 6x3, kyp 6x3.
 */
void oracle_stokes_reddy(int npts, const double* Gu, const double* Gp, const double* Np, const double* w,
                         int64_t nel, const int64_t* uconn, const int64_t* pconn, const double* uxy,
                         const double* pxy, double mu,
                         double* kxx, double* kyy, double* kxy, double* kxp, double* kyp) {
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < nel; ++e) {
        double gp[6], gu[12];
        double *a = kxx + e * 36, *b = kyy + e * 36, *cxy = kxy + e * 36, *dx = kxp + e * 18, *dy = kyp + e * 18;
        for (int i = 0; i < 36; ++i) { a[i] = 0; b[i] = 0; cxy[i] = 0; }
        for (int i = 0; i < 18; ++i) { dx[i] = 0; dy[i] = 0; }
        const int64_t* pc = pconn + e * 3;
        for (int q = 0; q < npts; ++q) {
            /* Jacobian from the pressure geometry; velocity gradients with that J */
            double J11 = 0, J12 = 0, J21 = 0, J22 = 0;
            const double* Gq = Gp + q * 6;
            for (int j = 0; j < 3; ++j) {
                double x = pxy[2 * pc[j]], y = pxy[2 * pc[j] + 1];
                J11 += x * Gq[2 * j]; J12 += x * Gq[2 * j + 1];
                J21 += y * Gq[2 * j]; J22 += y * Gq[2 * j + 1];
            }
            double det = J11 * J22 - J21 * J12;
            (void)gp;
            const double* Guq = Gu + q * 12;
            for (int j = 0; j < 6; ++j) {
                double g1 = Guq[2 * j], g2 = Guq[2 * j + 1];
                gu[2 * j] = (g1 * J22 - g2 * J21) / det;
                gu[2 * j + 1] = (-g1 * J12 + g2 * J11) / det;
            }
            double JxW = det * w[q];
            const double* Npq = Np + q * 3;
            for (int j = 0; j < 6; ++j)
                for (int i = 0; i < 6; ++i) {
                    a[i + 6 * j] += (mu * JxW) * (2 * gu[2 * i] * gu[2 * j] + gu[2 * i + 1] * gu[2 * j + 1]);
                    b[i + 6 * j] += (mu * JxW) * (gu[2 * i] * gu[2 * j] + 2 * gu[2 * i + 1] * gu[2 * j + 1]);
                    cxy[i + 6 * j] += (mu * JxW) * (gu[2 * i] * gu[2 * j + 1]);
                }
            for (int j = 0; j < 3; ++j)
                for (int i = 0; i < 6; ++i) {
                    dx[i + 6 * j] += (-JxW) * (gu[2 * i] * Npq[j]);
                    dy[i + 6 * j] += (-JxW) * (gu[2 * i + 1] * Npq[j]);
                }
        }
    }
}

/*
 * COO -> CSC with the semantics of SparseArrays.sparse(I, J, V, m, n), which
 * SysmatAssemblerSparse.finish! calls (src/Assemblers.jl:121-123):
 *   entries with equal (row, col) are summed in the order they were appended,
 *   explicitly assembled zeros stay in the pattern, rows sorted within a column.
 * Implemented as a stable counting sort by row, then a stable counting sort by
 * column, then a left-to-right sum over equal keys.
 * Returns nnz; colptr (ncol+1), rowval (nnz) and nzval (nnz) must hold at
 * least n entries.  I, J are 0-based.
 */
int64_t oracle_sparse(int64_t n, const int64_t* I, const int64_t* J, const double* V,
                      int64_t nrow, int64_t ncol, int64_t* colptr, int64_t* rowval, double* nzval) {
    int64_t* cnt = (int64_t*)calloc((size_t)(nrow > ncol ? nrow : ncol) + 1, sizeof(int64_t));
    int64_t* p1 = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n ? n : 1));
    int64_t* p2 = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n ? n : 1));
    /* stable sort by row */
    for (int64_t k = 0; k < n; ++k) cnt[I[k] + 1]++;
    for (int64_t r = 0; r < nrow; ++r) cnt[r + 1] += cnt[r];
    for (int64_t k = 0; k < n; ++k) p1[cnt[I[k]]++] = k;
    /* stable sort by column */
    memset(cnt, 0, sizeof(int64_t) * ((size_t)(nrow > ncol ? nrow : ncol) + 1));
    for (int64_t k = 0; k < n; ++k) cnt[J[k] + 1]++;
    for (int64_t c = 0; c < ncol; ++c) cnt[c + 1] += cnt[c];
    for (int64_t t = 0; t < n; ++t) { int64_t k = p1[t]; p2[cnt[J[k]]++] = k; }
    /* p2 is ordered by (col, row, input position); sum runs */
    int64_t nnz = 0;
    int64_t cur_col = -1;
    colptr[0] = 0;
    for (int64_t t = 0; t < n; ++t) {
        int64_t k = p2[t];
        int64_t c = J[k], r = I[k];
        while (cur_col < c) { ++cur_col; colptr[cur_col] = nnz; }
        if (nnz > colptr[c] && rowval[nnz - 1] == r) {
            nzval[nnz - 1] += V[k];
        } else {
            rowval[nnz] = r;
            nzval[nnz] = V[k];
            ++nnz;
        }
    }
    while (cur_col < ncol) { ++cur_col; colptr[cur_col] = nnz; }
    free(cnt); free(p1); free(p2);
    return nnz;
}

/* y = A x for CSR A (rowptr/col 0-based); A given as CSC of a symmetric matrix works too. */
static void csr_spmv(int64_t n, const int64_t* rp, const int64_t* ci, const double* v, const double* x, double* y) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double s = 0.0;
        for (int64_t k = rp[i]; k < rp[i + 1]; ++k) s += v[k] * x[ci[k]];
        y[i] = s;
    }
}

static double dotp(int64_t n, const double* a, const double* b) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/*
 * Jacobi-preconditioned conjugate gradients in FP64 on a CSR matrix.
 * Stops when ||b - A x||_2 / ||b||_2 <= rtol (recurrence residual) or maxit.
 * Returns the number of iterations; *relres gets the final recurrence residual.
 */
int oracle_pcg(int64_t n, const int64_t* rp, const int64_t* ci, const double* v, const double* b,
               double* x, double rtol, int maxit, double* relres) {
    double* r = (double*)malloc(sizeof(double) * (size_t)n);
    double* z = (double*)malloc(sizeof(double) * (size_t)n);
    double* p = (double*)malloc(sizeof(double) * (size_t)n);
    double* q = (double*)malloc(sizeof(double) * (size_t)n);
    double* dinv = (double*)malloc(sizeof(double) * (size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        double d = 0.0;
        for (int64_t k = rp[i]; k < rp[i + 1]; ++k)
            if (ci[k] == i) d = v[k];
        dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
    }
    csr_spmv(n, rp, ci, v, x, q);
    for (int64_t i = 0; i < n; ++i) { r[i] = b[i] - q[i]; z[i] = dinv[i] * r[i]; p[i] = z[i]; }
    double bn = sqrt(dotp(n, b, b));
    if (bn == 0.0) bn = 1.0;
    double rz = dotp(n, r, z);
    double rn = sqrt(dotp(n, r, r));
    int it = 0;
    while (it < maxit && rn / bn > rtol) {
        csr_spmv(n, rp, ci, v, p, q);
        double alpha = rz / dotp(n, p, q);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
            z[i] = dinv[i] * r[i];
        }
        double rz2 = dotp(n, r, z);
        double beta = rz2 / rz;
        rz = rz2;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        rn = sqrt(dotp(n, r, r));
        ++it;
    }
    *relres = rn / bn;
    free(r); free(z); free(p); free(q); free(dinv);
    return it;
}

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
