// porsol_oracle.cpp -- FP64 CPU oracle for the mimetic pressure / upstream transport path.
//
// TEST INFRASTRUCTURE ONLY.  A plain, serial C++ restatement of the reference algorithms
// of OPM/opm-porsol, used to check the GPU library.  Nothing in the product
// path links, loads or calls this file.  Each function cites the reference lines it
// restates.  Dense local algebra that the reference delegates to BLAS/LAPACK is written
// out here (Householder QR as in LAPACK xGEQR2/xORG2R, plain loops for SYRK/TRMM/GEMM).
// Linear-solver arithmetic the reference delegates to dune-istl (SeqILU0, CGSolver) is
// restated from the published algorithms: IKJ ILU(0) with the inverted pivot stored on
// the diagonal, and preconditioned CG that stops on the unpreconditioned residual
// 2-norm reduction.
#include "porsol_oracle.h"

#include <algorithm>
#include <cassert>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <unordered_map>
#include <utility>
#include <vector>

namespace {

struct Grid {
    int nc = 0;
    const int* facepos;
    const int* nb;
    const int* bid;
    const double* area;
    const double* fcent;
    const double* fnormal;
    const double* cvol;
    const double* ccent;
    explicit Grid(const orc_grid* g)
        : nc(g->num_cells), facepos(g->cell_facepos), nb(g->hf_neighbour), bid(g->hf_bid),
          area(g->hf_area), fcent(g->hf_centroid), fnormal(g->hf_normal),
          cvol(g->cell_volume), ccent(g->cell_centroid) {}
    int nf(int c) const { return facepos[c + 1] - facepos[c]; }
    int nhf() const { return facepos[nc]; }
    bool boundary(int hf) const { return nb[hf] < 0; }
};

// ---------------------------------------------------------------------------
// Householder QR of an m x n column-major matrix, replaced by its orthonormal
// factor Q (m x n).  Restates the LAPACK unblocked xGEQR2 + xORG2R pair that
// orthogonalizeColumns() calls (opm/porsol/common/Matrix.hpp:729-760).
// Returns 0 on success.
int householder_q(int m, int n, double* A)
{
    std::vector<double> tau(n, 0.0);
    for (int i = 0; i < n; ++i) {
        double alpha = A[i + i * m];
        double xnorm = 0.0;
        for (int r = i + 1; r < m; ++r) xnorm += A[r + i * m] * A[r + i * m];
        xnorm = std::sqrt(xnorm);
        double t = 0.0;
        if (xnorm != 0.0) {
            double beta = -std::copysign(std::hypot(alpha, xnorm), alpha);
            t = (beta - alpha) / beta;
            double scal = 1.0 / (alpha - beta);
            for (int r = i + 1; r < m; ++r) A[r + i * m] *= scal;
            alpha = beta;
        }
        tau[i] = t;
        A[i + i * m] = alpha;
        // apply H(i) = I - tau v v^T (v(i)=1) to A(i:m, i+1:n) from the left
        if (t != 0.0) {
            for (int j = i + 1; j < n; ++j) {
                double w = A[i + j * m];
                for (int r = i + 1; r < m; ++r) w += A[r + i * m] * A[r + j * m];
                w *= t;
                A[i + j * m] -= w;
                for (int r = i + 1; r < m; ++r) A[r + j * m] -= w * A[r + i * m];
            }
        }
    }
    // xORG2R: accumulate Q in place
    for (int i = n - 1; i >= 0; --i) {
        if (i < n - 1) {
            A[i + i * m] = 1.0;
            for (int j = i + 1; j < n; ++j) {
                double w = 0.0;
                for (int r = i; r < m; ++r) w += A[r + i * m] * A[r + j * m];
                w *= tau[i];
                for (int r = i; r < m; ++r) A[r + j * m] -= w * A[r + i * m];
            }
        }
        for (int r = i + 1; r < m; ++r) A[r + i * m] *= -tau[i];
        A[i + i * m] = 1.0 - tau[i];
        for (int r = 0; r < i; ++r) A[r + i * m] = 0.0;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// CSR helpers
struct Csr {
    int n = 0;
    std::vector<int> rowptr, col;
    std::vector<double> val;
    double& at(int i, int j)
    {
        auto b = col.begin() + rowptr[i], e = col.begin() + rowptr[i + 1];
        auto p = std::lower_bound(b, e, j);
        if (p == e || *p != j) throw std::runtime_error("oracle: entry outside sparsity pattern");
        return val[p - col.begin()];
    }
    double get(int i, int j) const
    {
        auto b = col.begin() + rowptr[i], e = col.begin() + rowptr[i + 1];
        auto p = std::lower_bound(b, e, j);
        if (p == e || *p != j) return 0.0;
        return val[p - col.begin()];
    }
};

// SeqILU0 (relaxation 1): IKJ ILU(0) on the pattern of A, pivots stored inverted.
struct Ilu0 {
    Csr lu;
    std::vector<int> diag;
    explicit Ilu0(const Csr& A) : lu(A), diag(A.n)
    {
        const int n = lu.n;
        for (int i = 0; i < n; ++i) {
            int d = -1;
            for (int k = lu.rowptr[i]; k < lu.rowptr[i + 1]; ++k)
                if (lu.col[k] == i) d = k;
            if (d < 0) throw std::runtime_error("oracle ILU0: diagonal entry missing");
            diag[i] = d;
        }
        for (int i = 0; i < n; ++i) {
            const int rb = lu.rowptr[i], re = lu.rowptr[i + 1];
            for (int ij = rb; ij < re && lu.col[ij] < i; ++ij) {
                const int j = lu.col[ij];
                lu.val[ij] *= lu.val[diag[j]];          // L_ij = a_ij * inv(a_jj)
                const double lij = lu.val[ij];
                int ik = ij + 1, jk = diag[j] + 1;
                const int je = lu.rowptr[j + 1];
                while (ik < re && jk < je) {
                    if (lu.col[ik] == lu.col[jk]) {
                        lu.val[ik] -= lij * lu.val[jk];
                        ++ik; ++jk;
                    } else if (lu.col[ik] < lu.col[jk]) {
                        ++ik;
                    } else {
                        ++jk;
                    }
                }
            }
            lu.val[diag[i]] = 1.0 / lu.val[diag[i]];
        }
    }
    void apply(double* v, const double* d) const
    {
        const int n = lu.n;
        for (int i = 0; i < n; ++i) {
            double r = d[i];
            for (int k = lu.rowptr[i]; k < diag[i]; ++k) r -= lu.val[k] * v[lu.col[k]];
            v[i] = r;
        }
        for (int i = n - 1; i >= 0; --i) {
            double r = v[i];
            for (int k = diag[i] + 1; k < lu.rowptr[i + 1]; ++k) r -= lu.val[k] * v[lu.col[k]];
            v[i] = lu.val[diag[i]] * r;
        }
    }
};

void spmv(const Csr& A, const double* x, double* y)
{
    for (int i = 0; i < A.n; ++i) {
        double s = 0.0;
        for (int k = A.rowptr[i]; k < A.rowptr[i + 1]; ++k) s += A.val[k] * x[A.col[k]];
        y[i] = s;
    }
}

double dot(int n, const double* a, const double* b)
{
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

// Optional record of when a CG run first reaches a looser residual reduction than its stopping
// tolerance (iteration and seconds since the CG started), so one solve to a tight tolerance also
// times the solve to the looser one.
struct Milestone {
    double tol = 0.0;
    int iteration = -1;
    double seconds = 0.0;
};

// Preconditioned CG as dune-istl's CGSolver::apply: x is the initial guess, b is
// overwritten by the defect; stop when ||b - A x||_2 < tol * ||b - A x0||_2 or < 1e-30.
// Returns true when converged.
bool pcg(const Csr& A, const Ilu0& M, std::vector<double>& x, std::vector<double> b,
         double tol, int maxit, int* iters, double* reduction, Milestone* ms = nullptr)
{
    const auto t_start = std::chrono::steady_clock::now();
    const int n = A.n;
    std::vector<double> p(n), q(n);
    spmv(A, x.data(), q.data());
    for (int i = 0; i < n; ++i) b[i] -= q[i];
    const double def0 = std::sqrt(dot(n, b.data(), b.data()));
    if (def0 < 1e-30) {
        *iters = 0;
        *reduction = 0.0;
        return true;
    }
    double def = def0;
    M.apply(p.data(), b.data());
    double rholast = dot(n, p.data(), b.data());
    int i = 1;
    bool converged = false;
    for (; i <= maxit; ++i) {
        spmv(A, p.data(), q.data());
        const double alpha = dot(n, p.data(), q.data());
        const double lambda = rholast / alpha;
        for (int k = 0; k < n; ++k) x[k] += lambda * p[k];
        for (int k = 0; k < n; ++k) b[k] -= lambda * q[k];
        def = std::sqrt(dot(n, b.data(), b.data()));
        if (ms && ms->iteration < 0 && def < def0 * ms->tol) {
            ms->iteration = i;
            ms->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        }
        if (def < def0 * tol || def < 1e-30) {
            converged = true;
            break;
        }
        M.apply(q.data(), b.data());
        const double rho = dot(n, q.data(), b.data());
        const double beta = rho / rholast;
        for (int k = 0; k < n; ++k) p[k] = beta * p[k] + q[k];
        rholast = rho;
    }
    if (i > maxit) i = maxit;
    *iters = i;
    *reduction = def / def0;
    return converged;
}

// ---------------------------------------------------------------------------
// IncompFlowSolverHybrid restatement.
enum FaceType { Internal, Dirichlet, Neumann, Periodic };

struct Pressure {
    Grid g;
    std::vector<int> cf;            // half-face -> dof (cellFaces_)
    int max_ncf = -1, num_internal = 0, total_faces = 0;
    std::unordered_map<int, std::pair<int, int>> bdry_id_map; // bid -> (cell, local face)
    std::vector<int> hf_partner_bid;
    std::vector<int> ppartner;      // ppartner_dof_
    Csr S;
    std::vector<double> rhs, soln;
    std::vector<int> binvpos;
    std::vector<double> Binv, gflux;
    std::vector<double> L, gv, F;   // L_, g_, F_
    std::vector<double> pressure, outflux;
    std::vector<double> totmob, mobdens;
    bool do_reg = true;
    std::vector<int> hf_type;       // FaceType per half-face of the last assembly

    Pressure(const orc_grid* og, const int* hf_flow_type, const int* partner_bid) : g(og)
    {
        const int nhf = g.nhf();
        hf_partner_bid.assign(partner_bid ? partner_bid : nullptr, partner_bid ? partner_bid + nhf : nullptr);
        if (!partner_bid) hf_partner_bid.assign(nhf, 0);
        enumerateGridDof();
        enumerateBCDof(hf_flow_type);
        buildPattern(hf_flow_type);
    }

    // IncompFlowSolverHybrid.hpp:956-1067
    void enumerateGridDof()
    {
        const int nc = g.nc;
        std::vector<int> cell(nc, -1), fpos, faces;
        fpos.push_back(0);
        for (int c = 0; c < nc; ++c) {
            cell[c] = c;
            for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf) {
                if (!g.boundary(hf)) {
                    const int c1 = g.nb[hf];
                    if (cell[c1] == -1) faces.push_back(c1);
                }
            }
            fpos.push_back(int(faces.size()));
            max_ncf = std::max(max_ncf, g.nf(c));
        }
        total_faces = num_internal = int(faces.size());
        cf.assign(g.nhf(), -1);
        for (int c = 0; c < nc; ++c) {
            for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf) {
                if (g.boundary(hf)) {
                    cf[hf] = total_faces++;
                } else {
                    int t = c, seek = g.nb[hf];
                    if (seek < t) std::swap(t, seek);
                    const int s = fpos[t], e = fpos[t + 1];
                    auto p = std::find(faces.begin() + s, faces.begin() + e, seek);
                    if (p == faces.begin() + e) throw std::runtime_error("oracle: inconsistent neighbour");
                    cf[hf] = int(p - faces.begin());
                }
            }
        }
        const int nhf = g.nhf();
        binvpos.assign(nc + 1, 0);
        for (int c = 0; c < nc; ++c) binvpos[c + 1] = binvpos[c] + g.nf(c) * g.nf(c);
        Binv.assign(binvpos[nc], 0.0);
        gflux.assign(nhf, 0.0);
        F.assign(nhf, 0.0);
        outflux.assign(nhf, 0.0);
    }

    // IncompFlowSolverHybrid.hpp:1071-1110
    void enumerateBCDof(const int* hf_flow_type)
    {
        bdry_id_map.clear();
        for (int c = 0; c < g.nc; ++c)
            for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf)
                if (g.boundary(hf) && hf_flow_type[hf] == ORC_BC_PERIODIC)
                    bdry_id_map.insert(std::make_pair(g.bid[hf], std::make_pair(c, hf - g.facepos[c])));
        ppartner.clear();
        if (!bdry_id_map.empty()) {
            ppartner.assign(total_faces, -1);
            for (int c = 0; c < g.nc; ++c)
                for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf)
                    if (g.boundary(hf) && hf_flow_type[hf] == ORC_BC_PERIODIC) {
                        const int dof1 = cf[hf];
                        const int dof2 = partnerDof(hf);
                        ppartner[dof1] = dof2;
                        ppartner[dof2] = dof1;
                    }
        }
    }

    int partnerDof(int hf) const
    {
        auto j = bdry_id_map.find(hf_partner_bid[hf]);
        if (j == bdry_id_map.end()) throw std::runtime_error("oracle: periodic partner not found");
        return cf[g.facepos[j->second.first] + j->second.second];
    }
    int partnerCell(int hf) const
    {
        auto j = bdry_id_map.find(hf_partner_bid[hf]);
        if (j == bdry_id_map.end()) throw std::runtime_error("oracle: periodic partner not found");
        return j->second.first;
    }

    // allocateConnections/setConnections, IncompFlowSolverHybrid.hpp:1115-1319
    void buildPattern(const int* hf_flow_type)
    {
        const int n = total_faces;
        std::vector<std::vector<int>> rows(n);
        for (int c = 0; c < g.nc; ++c)
            for (int i = g.facepos[c]; i < g.facepos[c + 1]; ++i)
                for (int j = g.facepos[c]; j < g.facepos[c + 1]; ++j) rows[cf[i]].push_back(cf[j]);
        if (!bdry_id_map.empty()) {
            for (int c = 0; c < g.nc; ++c)
                for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf) {
                    if (!(g.boundary(hf) && hf_flow_type[hf] == ORC_BC_PERIODIC)) continue;
                    const int dof1 = cf[hf];
                    const int c2 = partnerCell(hf);
                    const int dof2 = partnerDof(hf);
                    if (dof1 < dof2) {
                        for (int k = g.facepos[c2]; k < g.facepos[c2 + 1]; ++k) {
                            int ii = cf[k];
                            const int pp = ppartner[ii];
                            if (pp != -1 && pp != dof1 && pp < ii) ii = pp;
                            rows[dof1].push_back(ii);
                            rows[ii].push_back(dof1);
                            rows[dof2].push_back(ii);
                            rows[ii].push_back(dof2);
                        }
                    }
                }
        }
        for (int i = 0; i < n; ++i) rows[i].push_back(i);   // setrowsize(f, 1): diagonal always present
        S.n = n;
        S.rowptr.assign(n + 1, 0);
        for (int i = 0; i < n; ++i) {
            std::sort(rows[i].begin(), rows[i].end());
            rows[i].erase(std::unique(rows[i].begin(), rows[i].end()), rows[i].end());
            S.rowptr[i + 1] = S.rowptr[i] + int(rows[i].size());
        }
        S.col.resize(S.rowptr[n]);
        for (int i = 0; i < n; ++i) std::copy(rows[i].begin(), rows[i].end(), S.col.begin() + S.rowptr[i]);
        S.val.assign(S.rowptr[n], 0.0);
        rhs.assign(n, 0.0);
        soln.assign(n, 0.0);
        pressure.assign(g.nc, 0.0);
        gv.assign(g.nc, 0.0);
        L.assign(g.nc, 0.0);
    }

    // MimeticIPEvaluator::buildStaticContrib, MimeticIPEvaluator.hpp:201-270
    std::vector<double> perm;

    std::vector<double> Binv_static, gflux_static;
    double grav_[3] = {0.0, 0.0, 0.0};
    bool tensor_active = false;

    void computeInnerProducts(const double* K9, const double* grav)
    {
        perm.assign(K9, K9 + 9 * size_t(g.nc));
        for (int d = 0; d < 3; ++d) grav_[d] = grav[d];
        for (int c = 0; c < g.nc; ++c)
            cellInnerProduct(c, K9 + 9 * c, grav, &Binv[binvpos[c]], &gflux[g.facepos[c]]);
        Binv_static = Binv;
        gflux_static = gflux;
        tensor_active = false;
    }

    // Back to the static inner products after a tensor-mobility solve.
    void useStatic()
    {
        if (!tensor_active) return;
        Binv = Binv_static;
        gflux = gflux_static;
        tensor_active = false;
    }

    // MimeticIPAnisoRelpermEvaluator (MimeticIPAnisoRelpermEvaluator.hpp:207-400): per cell
    // Binv = W(lambda_t K) and gravity flux N (sum_i rho_i lambda_i) K g; lam, rlam are 9 per
    // cell row-major (rlam may be null: no gravity flux).  The assembly then uses unit mobility.
    void tensorInnerProducts(const double* lam, const double* rlam)
    {
        std::vector<double> gtmp, wtmp;
        for (int c = 0; c < g.nc; ++c) {
            const double* K = &perm[9 * size_t(c)];
            const double* L = lam + 9 * size_t(c);
            double LK[9];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) LK[3 * i + j] = L[3 * i] * K[j] + L[3 * i + 1] * K[3 + j] + L[3 * i + 2] * K[6 + j];
            const int nf = g.nf(c), f0 = g.facepos[c];
            gtmp.assign(nf, 0.0);
            cellInnerProduct(c, LK, grav_, &Binv[binvpos[c]], gtmp.data());
            if (rlam) {
                const double* R = rlam + 9 * size_t(c);
                double RK[9];
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) RK[3 * i + j] = R[3 * i] * K[j] + R[3 * i + 1] * K[3 + j] + R[3 * i + 2] * K[6 + j];
                wtmp.assign(size_t(nf) * nf, 0.0);
                cellInnerProduct(c, RK, grav_, wtmp.data(), &gflux[f0]);
            } else {
                for (int i = 0; i < nf; ++i) gflux[f0 + i] = 0.0;
            }
        }
        tensor_active = true;
    }

    // W (column-major nf x nf) and gravity flux of cell c for the row-major tensor K
    void cellInnerProduct(int c, const double* K, const double* grav, double* W, double* gfl) const
    {
        const int dim = 3;
        {
            const int nf = g.nf(c), f0 = g.facepos[c];
            double Kg[3];
            for (int i = 0; i < 3; ++i) Kg[i] = K[3 * i] * grav[0] + K[3 * i + 1] * grav[1] + K[3 * i + 2] * grav[2];
            std::vector<double> T1(nf * dim), T2(nf * dim), fa(nf);
            std::fill(W, W + nf * nf, 0.0);
            for (int i = 0; i < nf; ++i) {
                const int hf = f0 + i;
                W[i + i * nf] = 1.0;
                fa[i] = g.area[hf];
                double fc[3], fn[3];
                for (int d = 0; d < 3; ++d) {
                    fc[d] = (g.fcent[3 * hf + d] - g.ccent[3 * c + d]) * fa[i];
                    fn[d] = g.fnormal[3 * hf + d] * fa[i];
                }
                gfl[i] = fn[0] * Kg[0] + fn[1] * Kg[1] + fn[2] * Kg[2];
                for (int d = 0; d < 3; ++d) {
                    T1[i + d * nf] = fn[d];
                    T2[i + d * nf] = fc[d];
                }
            }
            householder_q(nf, dim, T2.data());
            // Binv <- I - Q Q^T (upper triangle, mirrored)
            for (int j = 0; j < nf; ++j)
                for (int i = 0; i <= j; ++i) {
                    double s = 0.0;
                    for (int l = 0; l < dim; ++l) s += T2[i + l * nf] * T2[j + l * nf];
                    W[i + j * nf] = W[i + j * nf] - s;
                }
            for (int j = 0; j < nf; ++j)
                for (int i = j + 1; i < nf; ++i) W[i + j * nf] = W[j + i * nf];
            // Binv <- diag(A) Binv diag(A)
            for (int j = 0; j < nf; ++j)
                for (int i = 0; i <= j; ++i) W[i + j * nf] = fa[i] * W[i + j * nf] * fa[j];
            for (int j = 0; j < nf; ++j)
                for (int i = j + 1; i < nf; ++i) W[i + j * nf] = W[j + i * nf];
            // T2 <- N K
            for (int i = 0; i < nf; ++i)
                for (int j = 0; j < dim; ++j) {
                    double s = 0.0;
                    for (int l = 0; l < dim; ++l) s += T1[i + l * nf] * K[3 * l + j];
                    T2[i + j * nf] = s;
                }
            // Binv <- (T2 N^T + t Binv)/vol, t = 6 tr(K)/d
            const double t = 6.0 * (K[0] + K[4] + K[8]) / dim;
            const double vol = g.cvol[c];
            const double a1 = 1.0 / vol, a2 = t / vol;
            for (int j = 0; j < nf; ++j)
                for (int i = 0; i < nf; ++i) {
                    double s = 0.0;
                    for (int l = 0; l < dim; ++l) s += T2[i + l * nf] * T1[j + l * nf];
                    W[i + j * nf] = a2 * W[i + j * nf] + a1 * s;
                }
        }
    }

    // assembleDynamic + setExternalContrib + buildCellContrib + addCellContrib,
    // IncompFlowSolverHybrid.hpp:1325-1382, 1736-1901
    void assemble(const double* tm, const double* md, const int* bct, const double* bcv, const double* src)
    {
        std::fill(S.val.begin(), S.val.end(), 0.0);
        std::fill(rhs.begin(), rhs.end(), 0.0);
        std::fill(gv.begin(), gv.end(), 0.0);
        std::fill(L.begin(), L.end(), 0.0);
        totmob.assign(tm, tm + g.nc);
        mobdens.assign(md, md + g.nc);
        hf_type.assign(g.nhf(), Internal);
        do_reg = true;
        std::vector<double> Sl, r, gfl;
        std::vector<int> ftype, ppart;
        std::vector<double> cval;
        for (int c = 0; c < g.nc; ++c) {
            const int nf = g.nf(c), f0 = g.facepos[c];
            r.assign(nf, 0.0);
            ftype.assign(nf, Internal);
            cval.assign(nf, 0.0);
            ppart.assign(nf, -1);
            gv[c] = src[c];
            for (int k = 0; k < nf; ++k) {
                const int hf = f0 + k;
                if (!g.boundary(hf)) continue;
                if (bct[hf] == ORC_BC_DIRICHLET) {
                    ftype[k] = Dirichlet;
                    cval[k] = bcv[hf];
                    do_reg = false;
                } else if (bct[hf] == ORC_BC_PERIODIC) {
                    ftype[k] = Periodic;
                    cval[k] = bcv[hf];
                    ppart[k] = partnerDof(hf);
                } else {
                    ftype[k] = Neumann;
                    r[k] = bcv[hf];
                }
            }
            for (int k = 0; k < nf; ++k) hf_type[f0 + k] = ftype[k];
            // getInverseMatrix: S = totmob * Binv
            Sl.assign(nf * nf, 0.0);
            const double* W = &Binv[binvpos[c]];
            for (int k = 0; k < nf * nf; ++k) Sl[k] = W[k] * tm[c];
            gfl.assign(nf, 0.0);
            for (int k = 0; k < nf; ++k) gfl[k] = gflux[f0 + k] * md[c];
            // buildCellContrib
            double* Fc = &F[f0];
            for (int j = 0; j < nf; ++j) {
                double s = 0.0;
                for (int i = 0; i < nf; ++i) s += Sl[i + j * nf];
                Fc[j] = s;
            }
            double Lc = 0.0;
            for (int j = 0; j < nf; ++j) Lc += Fc[j];
            L[c] = Lc;
            double gs = 0.0;
            for (int j = 0; j < nf; ++j) gs += gfl[j];
            gv[c] -= gs;
            for (int j = 0; j < nf; ++j) r[j] = gfl[j] - r[j];
            const double gl = gv[c] / L[c];
            for (int j = 0; j < nf; ++j) r[j] = 1.0 * r[j] + gl * Fc[j];
            const double a = -1.0 / L[c];
            for (int j = 0; j < nf; ++j)
                for (int i = 0; i <= j; ++i) Sl[i + j * nf] = Sl[i + j * nf] + Fc[i] * (a * Fc[j]);
            for (int j = 0; j < nf; ++j)
                for (int i = j + 1; i < nf; ++i) Sl[i + j * nf] = Sl[j + i * nf];
            // addCellContrib
            for (int rr = 0; rr < nf; ++rr) {
                int ii = cf[f0 + rr];
                const double Srr = Sl[rr + rr * nf];
                switch (ftype[rr]) {
                case Dirichlet:
                    S.at(ii, ii) = Srr;
                    rhs[ii] = Srr * cval[rr];
                    continue;
                case Periodic: {
                    const int pp = ppart[rr];
                    const double av = Srr, bv = av * cval[rr];
                    S.at(ii, ii) += av;
                    S.at(ii, pp) -= av;
                    rhs[ii] += bv;
                    S.at(pp, ii) -= av;
                    S.at(pp, pp) += av;
                    rhs[pp] -= bv;
                    ii = std::min(ii, pp);
                }
                    // fall through
                default:
                    for (int cc = 0; cc < nf; ++cc) {
                        int jj = cf[f0 + cc];
                        if (ftype[cc] == Dirichlet) {
                            rhs[ii] -= Sl[rr + cc * nf] * cval[cc];
                            continue;
                        }
                        if (ftype[cc] == Periodic) {
                            if (ppart[cc] < jj) {
                                rhs[ii] -= Sl[rr + cc * nf] * cval[cc];
                                jj = ppart[cc];
                            }
                        }
                        S.at(ii, jj) += Sl[rr + cc * nf];
                    }
                    break;
                }
                rhs[ii] += r[rr];
            }
        }
    }

    // solveLinearSystem / solveLinearSystemAMG (the Krylov part), :1387-1420, :1481-1541
    double t_factor = 0.0;
    int solve(double tol, int maxit, int dirichlet_guess, int* iters, double* red, Milestone* ms = nullptr)
    {
        if (do_reg) S.at(0, 0) *= 2;
        const auto tf0 = std::chrono::steady_clock::now();
        Ilu0 M(S);
        t_factor = std::chrono::duration<double>(std::chrono::steady_clock::now() - tf0).count();
        std::fill(soln.begin(), soln.end(), 0.0);
        if (dirichlet_guess) {
            for (int i = 0; i < S.n; ++i) {
                bool isD = true;
                for (int k = S.rowptr[i]; k < S.rowptr[i + 1]; ++k)
                    if (S.col[k] != i && S.val[k] != 0.0) isD = false;
                if (isD) soln[i] = rhs[i] / S.get(i, i);
            }
        }
        const bool ok = pcg(S, M, soln, rhs, tol, maxit > 0 ? maxit : S.n, iters, red, ms);
        return ok ? 0 : 1;
    }

    // Adjoint gradient of J = sum_c w_c (p_c - p*_c)^2 + sum_hf u_hf v_hf (v before
    // postProcessFluxes) with respect to ln s_c, K_c -> s_c K_c (mode 0), or ln k_{c,a} of a
    // diagonal tensor (mode 1, grad[3c + a]).  Zero gravity, no periodic faces, at least one
    // Dirichlet face.  The adjoint mu solves A mu = -dJ/dpi with the assembled matrix of the
    // last solve (mu = 0 on Dirichlet faces) by ILU0-CG; then per cell
    //   grad = dJ/dtheta|_pi + mu_c . (dS pi_c - db),  S = B - F F^T / L,  b = F g / L,
    // with dB = totmob W(K) (mode 0; W is linear in K) or totmob W(k_a e_a e_a^T) (mode 1).
    int adjoint(const double* wp, const double* pstar, const double* wv, int mode, double tol, double* grad,
                double* Jout, int* iters)
    {
        if (do_reg || (tensor_active && mode != 0)) return 2;
        for (int t : hf_type)
            if (t == Periodic) return 2;
        const int n = S.n;
        std::vector<double> b(n, 0.0), Sl, B, dB;
        std::vector<char> dir(n, 0);
        double J = 0.0;
        auto cell_S = [&](int c, std::vector<double>& out) {
            const int nf = g.nf(c), f0 = g.facepos[c];
            const double* W = &Binv[binvpos[c]];
            out.assign(nf * nf, 0.0);
            for (int j = 0; j < nf; ++j)
                for (int i = 0; i < nf; ++i)
                    out[i + j * nf] = W[i + j * nf] * totmob[c] - F[f0 + i] * F[f0 + j] / L[c];
        };
        for (int c = 0; c < g.nc; ++c) {
            const int nf = g.nf(c), f0 = g.facepos[c];
            cell_S(c, Sl);
            const double p = pressure[c], ps = pstar ? pstar[c] : 0.0;
            const double dev = wp ? wp[c] * (p - ps) : 0.0;
            J += dev * (p - ps);
            for (int i = 0; i < nf; ++i) {
                double spi = 0.0, su = 0.0;
                for (int j = 0; j < nf; ++j) {
                    spi += Sl[i + j * nf] * soln[cf[f0 + j]];
                    su += Sl[i + j * nf] * (wv ? wv[f0 + j] : 0.0);
                }
                const double u = wv ? wv[f0 + i] : 0.0;
                J += u * (F[f0 + i] * gv[c] / L[c] - spi);
                const double y = 2.0 * dev * F[f0 + i] / L[c] - su;
                if (hf_type[f0 + i] == Dirichlet) dir[cf[f0 + i]] = 1;
                else b[cf[f0 + i]] -= y;
            }
        }
        for (int i = 0; i < n; ++i)
            if (dir[i]) b[i] = 0.0;
        *Jout = J;
        Ilu0 M(S);
        std::vector<double> mu(n, 0.0);
        double red = 0.0;
        const bool ok = pcg(S, M, mu, b, tol, n, iters, &red);
        if (!ok) return 1;
        const double zero3[3] = {0.0, 0.0, 0.0};
        std::vector<double> gtmp;
        for (int c = 0; c < g.nc; ++c) {
            const int nf = g.nf(c), f0 = g.facepos[c];
            const double Lc = L[c], gc = gv[c], p = pressure[c];
            const double dev = wp ? wp[c] * (p - (pstar ? pstar[c] : 0.0)) : 0.0;
            std::vector<double> pi(nf), m(nf), Fc(F.begin() + f0, F.begin() + f0 + nf), u(nf);
            for (int i = 0; i < nf; ++i) {
                pi[i] = soln[cf[f0 + i]];
                m[i] = hf_type[f0 + i] == Dirichlet ? 0.0 : mu[cf[f0 + i]];
                u[i] = wv ? wv[f0 + i] : 0.0;
            }
            const int na = mode == 0 ? 1 : 3;
            for (int ax = 0; ax < na; ++ax) {
                dB.assign(nf * nf, 0.0);
                if (mode == 0) {
                    const double* W = &Binv[binvpos[c]];
                    for (int k = 0; k < nf * nf; ++k) dB[k] = W[k] * totmob[c];
                } else {
                    const double* K = &perm[9 * size_t(c)];
                    if (K[1] != 0.0 || K[2] != 0.0 || K[3] != 0.0 || K[5] != 0.0 || K[6] != 0.0 || K[7] != 0.0)
                        return 2;
                    double Ka[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                    Ka[4 * ax] = K[4 * ax];
                    gtmp.assign(nf, 0.0);
                    cellInnerProduct(c, Ka, zero3, dB.data(), gtmp.data());
                    for (int k = 0; k < nf * nf; ++k) dB[k] *= totmob[c];
                }
                std::vector<double> dF(nf, 0.0);
                double dL = 0.0, Fpi = 0.0, dFpi = 0.0;
                for (int i = 0; i < nf; ++i) {
                    for (int j = 0; j < nf; ++j) dF[i] += dB[i + j * nf];
                    dL += dF[i];
                    Fpi += Fc[i] * pi[i];
                    dFpi += dF[i] * pi[i];
                }
                const double dp = (dFpi - p * dL) / Lc;
                double gr = 2.0 * dev * dp;
                for (int i = 0; i < nf; ++i) {
                    double dBpi = 0.0;
                    for (int j = 0; j < nf; ++j) dBpi += dB[i + j * nf] * pi[j];
                    const double dv = p * dF[i] - dBpi + Fc[i] * dp;
                    const double dSpi = dBpi - (dF[i] * Fpi + Fc[i] * dFpi) / Lc + Fc[i] * Fpi * dL / (Lc * Lc);
                    const double db = gc * (dF[i] - Fc[i] * dL / Lc) / Lc;
                    gr += u[i] * dv + m[i] * (dSpi - db);
                }
                grad[na * size_t(c) + ax] = gr;
            }
        }
        return 0;
    }

    // computePressureAndFluxes, IncompFlowSolverHybrid.hpp:1672-1730
    void recover()
    {
        for (int c = 0; c < g.nc; ++c) {
            const int nf = g.nf(c), f0 = g.facepos[c];
            std::vector<double> pi(nf);
            double s = 0.0;
            for (int i = 0; i < nf; ++i) pi[i] = soln[cf[f0 + i]];
            for (int i = 0; i < nf; ++i) s += F[f0 + i] * pi[i];
            pressure[c] = (gv[c] + s) / L[c];
            for (int i = 0; i < nf; ++i) pi[i] = pressure[c] - pi[i];
            const double* W = &Binv[binvpos[c]];
            for (int i = 0; i < nf; ++i) {
                double v = 0.0;
                for (int j = 0; j < nf; ++j) v += (W[i + j * nf] * totmob[c]) * pi[j];
                outflux[f0 + i] = v;
            }
            for (int i = 0; i < nf; ++i) outflux[f0 + i] = gflux[f0 + i] * mobdens[c] + outflux[f0 + i];
        }
    }

    // postProcessFluxes + FaceFluxes, IncompFlowSolverHybrid.hpp:707-807
    double postProcess()
    {
        std::vector<double> fl(total_faces, 0.0);
        std::vector<int> vis(total_faces, 0);
        double maxmod = 0.0;
        auto put = [&](double flux, int f) {
            const double sign = vis[f] ? -1.0 : 1.0;
            fl[f] += sign * flux;
            ++vis[f];
        };
        auto get = [&](double& flux, int f) {
            const double sign = vis[f] ? -1.0 : 1.0;
            const double nf = 0.5 * sign * fl[f];
            maxmod = std::max(maxmod, std::fabs(flux - nf));
            flux = nf;
            ++vis[f];
        };
        for (int c = 0; c < g.nc; ++c)
            for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf) {
                const int f = cf[hf];
                if (g.boundary(hf)) {
                    if (ppartner.empty()) continue;
                    const int pf = ppartner[f];
                    if (pf != -1) {
                        put(outflux[hf], f);
                        put(outflux[hf], pf);
                    }
                } else {
                    put(outflux[hf], f);
                }
            }
        std::fill(vis.begin(), vis.end(), 0);
        for (int c = 0; c < g.nc; ++c)
            for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf) {
                const int f = cf[hf];
                if (g.boundary(hf)) {
                    if (ppartner.empty()) continue;
                    const int pf = ppartner[f];
                    if (pf != -1) {
                        get(outflux[hf], f);
                        double dummy = outflux[hf];
                        get(dummy, pf);
                    }
                } else {
                    get(outflux[hf], f);
                }
            }
        return maxmod;
    }
};

// ---------------------------------------------------------------------------
// Rock tables of RockJfunc (common/RockJfunc.hpp:63-216) with the cell -> rock map and the
// capillary functions of ReservoirPropertyCommon (common/ReservoirPropertyCommon_impl.hpp:
// 466-528, 740-781).  The reader's fix-ups are applied: krw starts at 0 and kro ends at 0
// (RockJfunc.hpp:200-207); s_min / s_max are the first / last saturation of the table.
// The table functions restate opm-core's NonuniformTableLinear, which is not part of the
// reference tree (unpinned): piecewise-linear interpolation with the end value outside the
// table; the derivative is the slope of the interval that holds the point (0 outside); the
// inverse interpolates the abscissa in the ordinate, read in increasing ordinate order.
double tab_value(const double* x, const double* y, int n, double v)
{
    if (v <= x[0]) return y[0];
    if (v >= x[n - 1]) return y[n - 1];
    int lo = 0, hi = n - 1;   // x[lo] <= v < x[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (x[mid] <= v) lo = mid;
        else hi = mid;
    }
    const double w = (v - x[lo]) / (x[hi] - x[lo]);
    return (1.0 - w) * y[lo] + w * y[hi];
}

double tab_slope(const double* x, const double* y, int n, double v)
{
    if (n < 2 || v < x[0] || v > x[n - 1]) return 0.0;
    int lo = 0, hi = n - 1;
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (x[mid] <= v) lo = mid;
        else hi = mid;
    }
    return x[hi] > x[lo] ? (y[hi] - y[lo]) / (x[hi] - x[lo]) : 0.0;
}

struct Rocks {
    int nrock = 0;
    std::vector<int> pos, cell;
    std::vector<double> s, krw, kro, J, Jx, sy;   // Jx/sy: the J table in increasing J order
    std::vector<double> skp;                      // per cell sqrt(tr K / (3 phi)) (J scaling)
    bool jscale = true;
    double sct = 1.0;

    // throws std::invalid_argument on malformed tables
    void set(const orc_rock_tables* rt, int nc, const double* K9, const double* poro)
    {
        nrock = rt->num_rocks;
        if (nrock < 1) throw std::invalid_argument("rock tables: no rock");
        pos.assign(rt->table_pos, rt->table_pos + nrock + 1);
        const int m = pos[nrock];
        s.assign(rt->s, rt->s + m);
        krw.assign(rt->krw, rt->krw + m);
        kro.assign(rt->kro, rt->kro + m);
        J.assign(rt->jfunc, rt->jfunc + m);
        Jx.resize(m);
        sy.resize(m);
        for (int r = 0; r < nrock; ++r) {
            const int a = pos[r], b = pos[r + 1];
            if (b - a < 1) throw std::invalid_argument("rock tables: empty table");
            for (int k = a + 1; k < b; ++k)
                if (!(s[k] >= s[k - 1])) throw std::invalid_argument("rock tables: saturations must increase");
            krw[a] = 0.0;
            kro[b - 1] = 0.0;
            const bool inc = J[b - 1] >= J[a];
            for (int k = a + 1; k < b; ++k)
                if (inc ? J[k] < J[k - 1] : J[k] > J[k - 1])
                    throw std::invalid_argument("rock tables: J must be monotone");
            for (int k = 0; k < b - a; ++k) {
                const int src = inc ? a + k : b - 1 - k;
                Jx[a + k] = J[src];
                sy[a + k] = s[src];
            }
        }
        cell.assign(rt->cell_rock, rt->cell_rock + nc);
        for (int c = 0; c < nc; ++c)
            if (cell[c] < 0 || cell[c] >= nrock) throw std::invalid_argument("rock tables: rock index out of range");
        jscale = rt->use_jfunction_scaling != 0;
        sct = rt->sigma_cos_theta;
        skp.assign(nc, 1.0);
        if (K9 && poro)
            for (int c = 0; c < nc; ++c)
                skp[c] = std::sqrt((K9[9 * c] + K9[9 * c + 4] + K9[9 * c + 8]) / (3 * poro[c]));
    }
    int n(int r) const { return pos[r + 1] - pos[r]; }
    double kr(int phase, int c, double sat) const
    {
        const int r = cell[c], a = pos[r];
        return tab_value(&s[a], phase == 0 ? &krw[a] : &kro[a], n(r), sat);
    }
    // RockJfunc::capPress (RockJfunc.hpp:94-107)
    double capPress(int c, double sat) const
    {
        const int r = cell[c], a = pos[r];
        const double j = tab_value(&s[a], &J[a], n(r), sat);
        return jscale ? j * sct / skp[c] : j;
    }
    // RockJfunc::capPressDeriv for perm = min_perm I and porosity max_poro (:110-123)
    double capPressDeriv(int r, double min_perm, double max_poro, double sat) const
    {
        const int a = pos[r];
        const double d = tab_slope(&s[a], &J[a], n(r), sat);
        return jscale ? d * sct / std::sqrt(3 * min_perm / (3 * max_poro)) : d;
    }
    // RockJfunc::satFromCapPress (:126-141)
    double satFromCapPress(int c, double pc) const
    {
        const int r = cell[c], a = pos[r];
        const double v = jscale ? pc * skp[c] / sct : pc;
        const double sat = tab_value(&Jx[a], &sy[a], n(r), v);
        return std::min(s[pos[r + 1] - 1], std::max(s[a], sat));
    }
};

// Transport restatement (EulerUpstream / EulerUpstreamResidual / cfl_calculator) for the
// scalar-mobility ReservoirPropertyCapillary: with rock tables the relative permeabilities
// and capillary pressure come from the tables above; without, kr1 = s^2, kr2 = (1-s)^2
// (ReservoirPropertyCapillary_impl.hpp:118-170) and pc = 1e5 (1-s)
// (ReservoirPropertyCommon_impl.hpp:466-476).
struct Fluid {
    double mu1, mu2, rho1, rho2;
    const Rocks* rk = nullptr;
    double mob(int phase, int c, double s) const
    {
        if (rk) return rk->kr(phase, c, s) / (phase == 0 ? mu1 : mu2);
        return phase == 0 ? (s * s) / mu1 : ((1 - s) * (1 - s)) / mu2;
    }
    double fracflow(int c, double s) const
    {
        const double l1 = mob(0, c, s), l2 = mob(1, c, s);
        return l1 / (l1 + l2);
    }
    double capPress(int c, double s) const { return rk ? rk->capPress(c, s) : 1e5 * (1 - s); }
};

struct TransportCtx {
    Grid g;
    const double* K9;
    Fluid fl;
    orc_transport_opts o;
    const int* st;
    const double* sv;
    const int* pbid;
    std::vector<int> bid_to_face;   // last periodic half-face seen with this bid
    std::vector<int> hf_cell;
    std::vector<double> cap;
    Rocks rocks;
    TransportCtx(const orc_grid* og, const double* K, const double* poro, const orc_fluid* f,
                 const orc_transport_opts* opts, const int* sat_type, const double* sat_value, const int* partner)
        : g(og), K9(K), st(sat_type), sv(sat_value), pbid(partner)
    {
        fl = Fluid{f->viscosity1, f->viscosity2, f->density1, f->density2};
        if (f->rocks) {
            rocks.set(f->rocks, g.nc, K, poro);
            fl.rk = &rocks;
        }
        o = *opts;
        int maxbid = 0;
        for (int hf = 0; hf < g.nhf(); ++hf) maxbid = std::max(maxbid, g.bid[hf]);
        bid_to_face.assign(maxbid + 1, -1);
        hf_cell.assign(g.nhf(), 0);
        for (int c = 0; c < g.nc; ++c)
            for (int hf = g.facepos[c]; hf < g.facepos[c + 1]; ++hf) {
                hf_cell[hf] = c;
                if (g.boundary(hf) && st[hf] == ORC_BC_PERIODIC) bid_to_face[g.bid[hf]] = hf;
            }
    }

    // EulerUpstreamResidual::estimateCapPressureGradient, EulerUpstreamResidual_impl.hpp:512-547
    void capGrad(int f, int nbf, double* out) const
    {
        if (g.boundary(f) && st[f] != ORC_BC_PERIODIC) {
            out[0] = out[1] = out[2] = 0.0;
            return;
        }
        const int c = hf_cell[f];
        const int nb = g.boundary(f) ? (f == nbf ? c : hf_cell[nbf]) : g.nb[f];
        double d0 = 0, d1 = 0, res[3], nrm = 0;
        for (int d = 0; d < 3; ++d) {
            const double a = g.ccent[3 * c + d] - g.fcent[3 * f + d];
            const double b = g.ccent[3 * nb + d] - g.fcent[3 * nbf + d];
            d0 += a * a;
            d1 += b * b;
            res[d] = g.ccent[3 * nb + d] - g.fcent[3 * nbf + d] + g.fcent[3 * f + d] - g.ccent[3 * c + d];
        }
        d0 = std::sqrt(d0);
        d1 = std::sqrt(d1);
        const double val = (cap[nb] - cap[c]) / (d0 + d1);
        for (int d = 0; d < 3; ++d) nrm += res[d] * res[d];
        nrm = std::sqrt(nrm);
        for (int d = 0; d < 3; ++d) out[d] = res[d] / nrm * val;
    }

    // UpdateForCell::operator(), EulerUpstreamResidual_impl.hpp:101-300, and
    // computeResidual :475-505 (serial order)
    void residual(const double* sat, const double* grav, const double* flux, const double* inj,
                  double* res)
    {
        const double delta_rho = fl.rho1 - fl.rho2;
        if (o.method_capillary) {
            cap.resize(g.nc);
            for (int c = 0; c < g.nc; ++c) cap[c] = fl.capPress(c, sat[c]);
        }
        std::fill(res, res + g.nc, 0.0);
        for (int c0 = 0; c0 < g.nc; ++c0) {
            int cell[2];
            double cs[2];
            cell[0] = c0;
            cs[0] = sat[c0];
            for (int f = g.facepos[c0]; f < g.facepos[c0 + 1]; ++f) {
                int nbface = f;
                double dS = 0.0;
                if (g.boundary(f)) {
                    if (st[f] == ORC_BC_PERIODIC) {
                        nbface = bid_to_face[pbid[f]];
                        cell[1] = hf_cell[nbface];
                        if (cell[0] > cell[1]) continue;
                        cs[1] = sat[cell[1]];
                    } else {
                        cell[1] = cell[0];
                        cs[1] = sv[f];
                    }
                } else {
                    cell[1] = g.nb[f];
                    if (cell[0] > cell[1]) continue;
                    cs[1] = sat[cell[1]];
                }
                const double A = g.area[f];
                const double q = flux[f];
                const double* n = &g.fnormal[3 * f];
                double Kav[9];
                for (int k = 0; k < 9; ++k) Kav[k] = 0.5 * (K9[9 * cell[0] + k] + K9[9 * cell[1] + k]);
                double gi[3];
                for (int i = 0; i < 3; ++i)
                    gi[i] = (Kav[3 * i] * grav[0] + Kav[3 * i + 1] * grav[1] + Kav[3 * i + 2] * grav[2]) * delta_rho;
                const double G = o.method_gravity ? A * (n[0] * gi[0] + n[1] * gi[1] + n[2] * gi[2]) : 0.0;
                const int triv = G >= 0.0 ? 0 : 1;
                const int ups = q >= 0.0 ? 0 : 1;
                double mu[2];
                mu[triv] = fl.mob(triv, cell[ups], cs[ups]);
                const double signG[2] = {-1.0, 1.0};
                const double gnt = signG[triv] * A * (n[0] * (mu[triv] * gi[0]) + n[1] * (mu[triv] * gi[1]) + n[2] * (mu[triv] * gi[2]));
                const int ups_nt = (q + gnt >= 0.0) ? 0 : 1;
                const int nontriv = (triv + 1) % 2;
                mu[nontriv] = fl.mob(nontriv, cell[ups_nt], cs[ups_nt]);
                const double mtot = mu[0] + mu[1];
                const double mtinv = 1.0 / mtot;
                const double asat = 0.5 * (cs[0] + cs[1]);
                const double m1 = 0.5 * (fl.mob(0, cell[0], asat) + fl.mob(0, cell[1], asat));
                const double m2 = 0.5 * (fl.mob(1, cell[0], asat) + fl.mob(1, cell[1], asat));
                const double matinv = 1.0 / (m1 + m2);
                if (o.method_viscous) {
                    double s = 0.0;
                    for (int d = 0; d < 3; ++d) s += n[d] * (mu[0] * (mtinv * (n[d] * q)));
                    dS += s;
                }
                if (o.method_gravity && cell[0] != cell[1]) {
                    double s = 0.0;
                    for (int d = 0; d < 3; ++d) s += n[d] * (mu[0] * (mtinv * (mu[1] * gi[d])));
                    dS += A * s;
                }
                if (o.method_capillary) {
                    double cg[3], ci[3];
                    capGrad(f, nbface, cg);
                    for (int i = 0; i < 3; ++i) ci[i] = Kav[3 * i] * cg[0] + Kav[3 * i + 1] * cg[1] + Kav[3 * i + 2] * cg[2];
                    double s = 0.0;
                    for (int d = 0; d < 3; ++d) s += n[d] * (m1 * (matinv * (m2 * ci[d])));
                    dS += A * s;
                }
                if (cell[0] != cell[1]) {
                    res[cell[0]] -= dS;
                    res[cell[1]] += dS;
                } else {
                    res[cell[0]] -= dS;
                }
            }
            double rate = inj ? inj[c0] : 0.0;
            if (rate < 0.0) rate *= fl.fracflow(c0, cs[0]);
            res[c0] += rate;
        }
    }
};

// ReservoirPropertyCapillary::computeSingleRockCflFactors (ReservoirPropertyCapillary_impl.hpp:
// 213-250): 257-point sampling of the fractional flow, the gravity flow function and (with a
// rock table) the capillary-pressure derivative; rock -1 = no table.
void single_rock_cfl(const Fluid& fl, int rock, double min_perm, double max_poro, double* out)
{
    const int N = 257;
    const double delta = 1.0 / double(N - 1);
    auto ff = [&](double s, double& f1, double& fg) {
        double l1, l2;
        if (rock < 0) {
            l1 = (s * s) / fl.mu1;
            l2 = ((1 - s) * (1 - s)) / fl.mu2;
        } else {
            const Rocks& R = *fl.rk;
            const int a = R.pos[rock], n = R.n(rock);
            l1 = tab_value(&R.s[a], &R.krw[a], n, s) / fl.mu1;
            l2 = tab_value(&R.s[a], &R.kro[a], n, s) / fl.mu2;
        }
        f1 = l1 / (l1 + l2);
        fg = l1 * l2 / (l1 + l2);
    };
    double last1, lastg, md1 = -1e100, mdg = -1e100;
    ff(0.0, last1, lastg);
    double maxffg = lastg;
    double mdpc = rock < 0 ? 0.0 : std::fabs(fl.rk->capPressDeriv(rock, min_perm, max_poro, 0.0));
    for (int i = 1; i < N; ++i) {
        const double s = double(i) * delta;
        double f1, fg;
        ff(s, f1, fg);
        md1 = std::max(md1, std::fabs(f1 - last1) / delta);
        mdg = std::max(mdg, std::fabs(fg - lastg) / delta);
        maxffg = std::max(maxffg, fg);
        if (rock >= 0) mdpc = std::max(mdpc, std::fabs(fl.rk->capPressDeriv(rock, min_perm, max_poro, s)));
        last1 = f1;
        lastg = fg;
    }
    out[0] = 1.0 / md1;
    out[1] = 1.0 / mdg;
    out[2] = maxffg * mdpc;
}

// ReservoirPropertyCapillary::computeCflFactors (:255-282): per rock the smallest mean diagonal
// permeability and the largest porosity of its cells; the most restrictive factors win.
void cfl_factors(const Fluid& fl, int nc, const double* K9, const double* poro, double* out)
{
    if (!fl.rk) {
        single_rock_cfl(fl, -1, 0.0, 0.0, out);
        return;
    }
    const Rocks& R = *fl.rk;
    std::vector<double> min_perm(R.nrock, 1e100), max_poro(R.nrock, 0.0);
    for (int c = 0; c < nc; ++c) {
        const int r = R.cell[c];
        min_perm[r] = std::min(min_perm[r], (K9[9 * c] + K9[9 * c + 4] + K9[9 * c + 8]) / 3.0);
        max_poro[r] = std::max(max_poro[r], poro[c]);
    }
    out[0] = 1e100;
    out[1] = 1e100;
    out[2] = 0.0;
    for (int r = 0; r < R.nrock; ++r) {
        double f[3];
        single_rock_cfl(fl, r, min_perm[r], max_poro[r], f);
        out[0] = std::min(out[0], f[0]);
        out[1] = std::min(out[1], f[1]);
        out[2] = std::max(out[2], f[2]);
    }
}

// computeCflTime, EulerUpstream_impl.hpp:265-331, and cfl_calculator, CflCalculator.hpp:55-170
double cfl_time(const Grid& g, const double* K9, const double* poro, const Fluid& fl,
                const orc_transport_opts& o, const double* flux, const double* grav)
{
    double fac[3];
    cfl_factors(fl, g.nc, K9, poro, fac);
    double dtv = 1e99, dtg = 1e99, dtc = 1e99;
    if (o.method_viscous && o.use_cfl_viscous) {
        double dt = 1e100;
        for (int c = 0; c < g.nc; ++c) {
            double fp = 0.0, fn = 0.0;
            for (int f = g.facepos[c]; f < g.facepos[c + 1]; ++f) {
                if (flux[f] > 0) fp += flux[f];
                else fn -= flux[f];
            }
            const double fx = std::max(fn, fp);
            const double loc = (fac[0] * g.cvol[c] * poro[c]) / fx;
            if (loc == 0.0) throw std::runtime_error("Cfl computation gave dt = 0.0");
            if (loc < dt) dt = loc;
        }
        dtv = dt;
    }
    if (o.method_gravity && o.use_cfl_gravity) {
        double dt = 1e100;
        const double drho = fl.rho1 - fl.rho2;
        for (int c = 0; c < g.nc; ++c) {
            double fx = 0.0;
            for (int f = g.facepos[c]; f < g.facepos[c + 1]; ++f) {
                double Kl[9];
                const int c1 = g.nb[f];
                for (int k = 0; k < 9; ++k)
                    Kl[k] = g.boundary(f) ? K9[9 * c + k] : 0.5 * (K9[9 * c + k] + K9[9 * c1 + k]);
                const double* n = &g.fnormal[3 * f];
                double gf = 0.0;
                for (int k = 0; k < 3; ++k)
                    for (int q = 0; q < 3; ++q) gf += n[q] * (Kl[3 * q + k] * grav[k] * drho);
                gf *= g.area[f];
                if (gf > 0) fx += gf;
            }
            const double loc = (fac[1] * g.cvol[c] * poro[c]) / fx;
            if (loc < dt) dt = loc;
        }
        dtg = dt;
    }
    if (o.method_capillary && o.use_cfl_capillary) {
        double dt = 1e100;
        for (int c = 0; c < g.nc; ++c)
            for (int f = g.facepos[c]; f < g.facepos[c + 1]; ++f) {
                double Kl[9];
                const int c1 = g.nb[f];
                for (int k = 0; k < 9; ++k)
                    Kl[k] = g.boundary(f) ? K9[9 * c + k] : 0.5 * (K9[9 * c + k] + K9[9 * c1 + k]);
                // inverse3x3 (MatrixInverse.hpp:85) by cofactors
                const double det = Kl[0] * (Kl[4] * Kl[8] - Kl[5] * Kl[7]) - Kl[1] * (Kl[3] * Kl[8] - Kl[5] * Kl[6]) +
                                   Kl[2] * (Kl[3] * Kl[7] - Kl[4] * Kl[6]);
                double Ki[9];
                Ki[0] = (Kl[4] * Kl[8] - Kl[5] * Kl[7]) / det;
                Ki[1] = (Kl[2] * Kl[7] - Kl[1] * Kl[8]) / det;
                Ki[2] = (Kl[1] * Kl[5] - Kl[2] * Kl[4]) / det;
                Ki[3] = (Kl[5] * Kl[6] - Kl[3] * Kl[8]) / det;
                Ki[4] = (Kl[0] * Kl[8] - Kl[2] * Kl[6]) / det;
                Ki[5] = (Kl[2] * Kl[3] - Kl[0] * Kl[5]) / det;
                Ki[6] = (Kl[3] * Kl[7] - Kl[4] * Kl[6]) / det;
                Ki[7] = (Kl[1] * Kl[6] - Kl[0] * Kl[7]) / det;
                Ki[8] = (Kl[0] * Kl[4] - Kl[1] * Kl[3]) / det;
                double x[3];
                for (int d = 0; d < 3; ++d) x[d] = g.fcent[3 * f + d] - g.ccent[3 * c + d];
                double s = 0.0;
                for (int i = 0; i < 3; ++i) s += x[i] * (Ki[3 * i] * x[0] + Ki[3 * i + 1] * x[1] + Ki[3 * i + 2] * x[2]);
                dt = std::min(dt, s / fac[2]);
            }
        dtc = dt;
    }
    double dt = std::min(std::min(dtv, dtg), dtc);
    return dt * o.courant_number;
}

struct SatRangeError {};

// Root bracketing and regula falsi as ImplicitCapillarity uses them from opm-core's
// RootFinders (not part of the reference tree; unpinned), restated from the published
// methods.  bracket_zero steps away from x0 by dx, alternating sides and doubling the step,
// until the sign of f changes (at most 100 trials); regula_falsi is false position with the
// Pegasus modification (Dowell & Jarratt, BIT 12 (1972) 503-508) and stops at |f| <= tol.
// Error codes: 4 = no sign change found, 5 = more than max_iter iterations.
struct RootError {
    int code;
};

template <class F>
void bracket_zero(F& f, double x0, double dx, double& a, double& b)
{
    const double f0 = f(x0);
    double step = dx;
    for (int i = 0; i < 100; ++i) {
        const double x = x0 + step;
        if (f0 * f(x) <= 0.0) {
            a = std::min(x0, x);
            b = std::max(x0, x);
            return;
        }
        step = -2.0 * step;
    }
    throw RootError{4};
}

template <class F>
double regula_falsi(F& f, double a, double b, int max_iter, double tol, int* iters)
{
    *iters = 0;
    double x0 = a, f0 = f(x0);
    if (std::fabs(f0) <= tol) return x0;
    double x1 = b, f1 = f(x1);
    if (std::fabs(f1) <= tol) return x1;
    if (f0 * f1 > 0.0) throw RootError{4};
    for (int it = 1; it <= max_iter; ++it) {
        const double x = x1 - f1 * (x1 - x0) / (f1 - f0);
        const double fx = f(x);
        *iters = it;
        if (std::fabs(fx) <= tol) return x;
        if ((fx < 0.0) != (f1 < 0.0)) {
            x0 = x1;
            f0 = f1;
        } else {
            f0 *= f1 / (f1 + fx);
        }
        x1 = x;
        f1 = fx;
    }
    throw RootError{5};
}

}  // namespace

// ===========================================================================
extern "C" {

void* orc_create(const orc_grid* g, const int* hf_flow_type, const int* hf_partner_bid)
{
    try {
        return new Pressure(g, hf_flow_type, hf_partner_bid);
    } catch (...) {
        return nullptr;
    }
}
void orc_destroy(void* h) { delete static_cast<Pressure*>(h); }
int orc_num_dofs(void* h) { return static_cast<Pressure*>(h)->total_faces; }
int orc_nnz(void* h) { return int(static_cast<Pressure*>(h)->S.col.size()); }
int orc_max_ncf(void* h) { return static_cast<Pressure*>(h)->max_ncf; }
int orc_num_internal_faces(void* h) { return static_cast<Pressure*>(h)->num_internal; }

void orc_get_structure(void* h, int* cellfaces, int* rowptr, int* colind, int* ppartner)
{
    Pressure* P = static_cast<Pressure*>(h);
    if (cellfaces) std::copy(P->cf.begin(), P->cf.end(), cellfaces);
    if (rowptr) std::copy(P->S.rowptr.begin(), P->S.rowptr.end(), rowptr);
    if (colind) std::copy(P->S.col.begin(), P->S.col.end(), colind);
    if (ppartner) {
        if (P->ppartner.empty()) std::fill(ppartner, ppartner + P->total_faces, -1);
        else std::copy(P->ppartner.begin(), P->ppartner.end(), ppartner);
    }
}

void orc_compute_inner_products(void* h, const double* K9, const double* grav)
{
    static_cast<Pressure*>(h)->computeInnerProducts(K9, grav);
}

void orc_get_inner_products(void* h, double* Binv, double* gflux)
{
    Pressure* P = static_cast<Pressure*>(h);
    if (Binv) std::copy(P->Binv.begin(), P->Binv.end(), Binv);
    if (gflux) std::copy(P->gflux.begin(), P->gflux.end(), gflux);
}

void orc_assemble(void* h, const double* totmob, const double* mobdens, const int* bct, const double* bcv,
                  const double* src)
{
    static_cast<Pressure*>(h)->useStatic();
    static_cast<Pressure*>(h)->assemble(totmob, mobdens, bct, bcv, src);
}

int orc_solve_tensor(void* h, const double* lam, const double* rlam, const int* bct, const double* bcv,
                     const double* src, double tol, int maxit, int* iterations, double* reduction)
{
    Pressure* P = static_cast<Pressure*>(h);
    P->tensorInnerProducts(lam, rlam);
    const int nc = P->g.nc;
    std::vector<double> one(nc, 1.0), md(nc, rlam ? 1.0 : 0.0);
    P->assemble(one.data(), md.data(), bct, bcv, src);
    int it = 0;
    double red = 0.0;
    const int rc = P->solve(tol, maxit, 0, &it, &red);
    if (iterations) *iterations = it;
    if (reduction) *reduction = red;
    P->recover();
    return rc;
}

void orc_get_system(void* h, double* Svals, double* rhs, double* F, double* L, double* g, int* do_reg)
{
    Pressure* P = static_cast<Pressure*>(h);
    if (Svals) std::copy(P->S.val.begin(), P->S.val.end(), Svals);
    if (rhs) std::copy(P->rhs.begin(), P->rhs.end(), rhs);
    if (F) std::copy(P->F.begin(), P->F.end(), F);
    if (L) std::copy(P->L.begin(), P->L.end(), L);
    if (g) std::copy(P->gv.begin(), P->gv.end(), g);
    if (do_reg) *do_reg = P->do_reg ? 1 : 0;
}

int orc_solve(void* h, const double* totmob, const double* mobdens, const int* bct, const double* bcv,
              const double* src, double tol, int maxit, int dirichlet_guess, int* iterations, double* reduction)
{
    return orc_solve_timed(h, totmob, mobdens, bct, bcv, src, tol, maxit, dirichlet_guess, iterations, reduction,
                           nullptr);
}

int orc_solve_timed(void* h, const double* totmob, const double* mobdens, const int* bct, const double* bcv,
                    const double* src, double tol, int maxit, int dirichlet_guess, int* iterations,
                    double* reduction, double* seconds3)
{
    return orc_solve_milestone(h, totmob, mobdens, bct, bcv, src, tol, maxit, dirichlet_guess, iterations, reduction,
                               seconds3, 0.0, nullptr, nullptr);
}

int orc_solve_milestone(void* h, const double* totmob, const double* mobdens, const int* bct, const double* bcv,
                        const double* src, double tol, int maxit, int dirichlet_guess, int* iterations,
                        double* reduction, double* seconds3, double milestone_tol, int* milestone_iteration,
                        double* milestone_seconds)
{
    using clk = std::chrono::steady_clock;
    Milestone ms;
    ms.tol = milestone_tol;
    Pressure* P = static_cast<Pressure*>(h);
    const auto t0 = clk::now();
    P->useStatic();
    P->assemble(totmob, mobdens, bct, bcv, src);
    const auto t1 = clk::now();
    int it = 0;
    double red = 0.0;
    const int rc = P->solve(tol, maxit, dirichlet_guess, &it, &red, milestone_tol > 0.0 ? &ms : nullptr);
    const auto t2 = clk::now();
    if (milestone_iteration) *milestone_iteration = ms.iteration;
    if (milestone_seconds) *milestone_seconds = ms.seconds;
    if (iterations) *iterations = it;
    if (reduction) *reduction = red;
    P->recover();
    const auto t3 = clk::now();
    if (seconds3) {
        seconds3[0] = std::chrono::duration<double>(t1 - t0).count() + std::chrono::duration<double>(t3 - t2).count();
        seconds3[1] = P->t_factor;
        seconds3[2] = std::chrono::duration<double>(t2 - t1).count() - P->t_factor;
    }
    return rc;
}

void orc_get_solution(void* h, double* pressure, double* outflux, double* facepressure)
{
    Pressure* P = static_cast<Pressure*>(h);
    if (pressure) std::copy(P->pressure.begin(), P->pressure.end(), pressure);
    if (outflux) std::copy(P->outflux.begin(), P->outflux.end(), outflux);
    if (facepressure) std::copy(P->soln.begin(), P->soln.end(), facepressure);
}

double orc_post_process_fluxes(void* h) { return static_cast<Pressure*>(h)->postProcess(); }

int orc_adjoint_gradient(void* h, const double* cell_weight, const double* cell_target, const double* hf_weight,
                         int mode, double tol, double* grad, double* objective, int* iterations)
{
    return static_cast<Pressure*>(h)->adjoint(cell_weight, cell_target, hf_weight, mode, tol, grad, objective,
                                              iterations);
}

int orc_ilu0_cg(int n, const int* rowptr, const int* colind, const double* vals, const double* b, double* x,
                double tol, int maxit, int* iterations, double* reduction)
{
    Csr A;
    A.n = n;
    A.rowptr.assign(rowptr, rowptr + n + 1);
    A.col.assign(colind, colind + rowptr[n]);
    A.val.assign(vals, vals + rowptr[n]);
    Ilu0 M(A);
    std::vector<double> xv(x, x + n), bv(b, b + n);
    int it = 0;
    double red = 0.0;
    const bool ok = pcg(A, M, xv, bv, tol, maxit > 0 ? maxit : n, &it, &red);
    std::copy(xv.begin(), xv.end(), x);
    if (iterations) *iterations = it;
    if (reduction) *reduction = red;
    return ok ? 0 : 1;
}

void orc_cfl_factors(const orc_fluid* f, int nc, const double* K9, const double* poro, double* out3)
{
    Fluid fl{f->viscosity1, f->viscosity2, f->density1, f->density2};
    Rocks R;
    if (f->rocks) {
        R.set(f->rocks, nc, K9, poro);
        fl.rk = &R;
    }
    cfl_factors(fl, nc, K9, poro, out3);
}

double orc_transport_cfl(const orc_grid* og, const double* K9, const double* poro, const orc_fluid* f,
                         const orc_transport_opts* opts, const double* flux, const double* grav)
{
    Grid g(og);
    Fluid fl{f->viscosity1, f->viscosity2, f->density1, f->density2};
    Rocks R;
    if (f->rocks) {
        R.set(f->rocks, g.nc, K9, poro);
        fl.rk = &R;
    }
    try {
        return cfl_time(g, K9, poro, fl, *opts, flux, grav);
    } catch (...) {
        return 0.0;
    }
}

void orc_transport_residual(const orc_grid* g, const double* K9, const double* poro, const orc_fluid* fl,
                            const orc_transport_opts* opts, const int* st, const double* sv, const int* pbid,
                            const double* flux, const double* inj, const double* sat, const double* grav,
                            double* residual)
{
    TransportCtx T(g, K9, poro, fl, opts, st, sv, pbid);
    T.residual(sat, grav, flux, inj, residual);
}

// EulerUpstream::transportSolve, EulerUpstream_impl.hpp:153-218; smallTimeStep :357-385;
// checkAndPossiblyClampSat :337-349
int orc_transport_solve(const orc_grid* og, const double* K9, const double* poro, const orc_fluid* f,
                        const orc_transport_opts* opts, const int* st, const double* sv, const int* pbid,
                        const double* flux, const double* inj, double* sat, double time, const double* grav,
                        int* nsteps, int* repeats)
{
    Grid g(og);
    std::unique_ptr<TransportCtx> Tp;
    try {
        Tp.reset(new TransportCtx(og, K9, poro, f, opts, st, sv, pbid));
    } catch (const std::invalid_argument&) {
        return 6;
    }
    TransportCtx& T = *Tp;
    const orc_transport_opts& o = *opts;
    double cfl_dt;
    try {
        cfl_dt = cfl_time(g, K9, poro, T.fl, o, flux, grav);
    } catch (...) {
        return 3;
    }
    int n;
    if (cfl_dt > time) {
        n = o.minimum_small_steps;
    } else {
        const double steps = std::min<double>(std::ceil(time / cfl_dt), double(std::numeric_limits<int>::max()));
        n = int(steps);
        n = std::max(n, o.minimum_small_steps);
        n = std::min(n, o.maximum_small_steps);
    }
    double dt = time / n;
    std::vector<double> porevol(g.nc), s0(sat, sat + g.nc), res(g.nc);
    for (int c = 0; c < g.nc; ++c) porevol[c] = g.cvol[c] * poro[c];
    int rep = 0;
    const int max_repeats = 10;
    while (true) {
        bool failed = false;
        for (int q = 0; q < n && !failed; ++q) {
            T.residual(sat, grav, flux, inj, res.data());
            for (int i = 0; i < g.nc; ++i) sat[i] += dt * res[i] / porevol[i];
            if (o.check_sat || o.clamp_sat) {
                for (int i = 0; i < g.nc; ++i) {
                    if (sat[i] > 1.0 || sat[i] < 0.0) {
                        if (o.clamp_sat) sat[i] = std::max(std::min(sat[i], 1.0), 0.0);
                        else if (sat[i] > 1.001 || sat[i] < -0.001) {
                            failed = true;
                            break;
                        }
                    }
                }
            }
        }
        if (!failed) break;
        ++rep;
        if (rep > max_repeats) {
            if (nsteps) *nsteps = n;
            if (repeats) *repeats = rep;
            return 2;
        }
        n *= 2;
        dt = time / n;
        std::copy(s0.begin(), s0.end(), sat);
    }
    if (nsteps) *nsteps = n;
    if (repeats) *repeats = rep;
    return 0;
}

// ImplicitCapillarity::transportSolve (euler/ImplicitCapillarity_impl.hpp:138-226) with
// MatchSaturatedVolumeFunctor (euler/MatchSaturatedVolumeFunctor.hpp:49-112).  The pressure
// handle must hold the grid, the flow-BC topology and the inner products for zero gravity
// (the reference's psolver_ is initialised with zero gravity, :80-83).  Without rock tables
// saturationFromCapillaryPressure is 0 (ReservoirPropertyCommon_impl.hpp:518-528).
int orc_capillary_solve(void* ph, const orc_grid* og, const double* K9, const double* poro, const orc_fluid* f,
                        const orc_capillary_opts* co, const int* st, const double* sv, const int* pbid,
                        const int* bct, const double* bcv, const double* flux, const double* inj, double* sat,
                        const double* grav, double* shift, int* root_iterations, int* cg_iterations)
{
    Pressure* P = static_cast<Pressure*>(ph);
    Grid g(og);
    const int nc = g.nc, nhf = g.nhf();
    orc_transport_opts to{};
    to.method_viscous = co->method_viscous;
    to.method_gravity = co->method_gravity;
    to.method_capillary = 0;
    std::unique_ptr<TransportCtx> Tp;
    try {
        Tp.reset(new TransportCtx(og, K9, poro, f, &to, st, sv, pbid));
    } catch (const std::invalid_argument&) {
        return 6;
    }
    TransportCtx& T = *Tp;
    // capillary mobilities lambda_1 lambda_2 / (lambda_1 + lambda_2), threshold 1e-10 (:148-165)
    std::vector<double> capmob(nc);
    for (int c = 0; c < nc; ++c) {
        const double m1 = T.fl.mob(0, c, sat[c]), m2 = T.fl.mob(1, c, sat[c]);
        const double mtinv = 1.0 / (m1 + m2);
        capmob[c] = std::max((m1 * mtinv) * m2, 1e-10);
    }
    // periodic flow conditions get a zero jump (:168-174)
    std::vector<double> bv(bcv, bcv + nhf);
    for (int hf = 0; hf < nhf; ++hf)
        if (g.boundary(hf) && bct[hf] == ORC_BC_PERIODIC) bv[hf] = 0.0;
    // injection rates from the viscous/gravity residual (:176-183)
    std::vector<double> res(nc);
    T.residual(sat, grav, flux, inj, res.data());
    for (int c = 0; c < nc; ++c) res[c] = -res[c];
    // capillary pressure: a pressure solve with the fixed mobilities, phase densities (1, 0) (:186-193,
    // ReservoirPropertyFixedMobility.hpp:55-74)
    P->useStatic();
    P->assemble(capmob.data(), capmob.data(), bct, bv.data(), res.data());
    int it = 0;
    double red = 0.0;
    if (P->solve(co->residual_tolerance, 0, co->linsolver_type != 0, &it, &red) != 0) return 1;
    P->recover();
    if (cg_iterations) *cg_iterations = it;
    const std::vector<double> cp = P->pressure;
    // MatchSaturatedVolumeFunctor
    std::vector<double> snew(nc);
    double pv_sum = 0.0, sv0 = 0.0;
    for (int c = 0; c < nc; ++c) {
        const double pv = g.cvol[c] * poro[c];
        pv_sum += pv;
        sv0 += pv * sat[c];
    }
    auto fun = [&](double dp) {
        double pvs = 0.0, svs = 0.0;
        for (int c = 0; c < nc; ++c) {
            snew[c] = T.fl.rk ? T.fl.rk->satFromCapPress(c, cp[c] + dp) : 0.0;
            const double pv = g.cvol[c] * poro[c];
            pvs += pv;
            svs += pv * snew[c];
        }
        return (svs - sv0) / pvs;
    };
    (void)pv_sum;
    const double lo = *std::min_element(cp.begin(), cp.end()), hi = *std::max_element(cp.begin(), cp.end());
    double a = 1e100, b = -1e100, x;
    int rit = 0;
    try {
        bracket_zero(fun, 0.0, hi - lo, a, b);
        x = regula_falsi(fun, a, b, 40, 1e-12, &rit);
    } catch (const RootError& e) {
        return e.code;
    }
    if (shift) *shift = x;
    if (root_iterations) *root_iterations = rit;
    const double w = co->update_relaxation;
    for (int c = 0; c < nc; ++c) sat[c] = (1.0 - w) * sat[c] + w * snew[c];
    // relaxation (:213-217), checkAndPossiblyClampSat (:234-247)
    if (co->check_sat || co->clamp_sat) {
        for (int c = 0; c < nc; ++c) {
            if (sat[c] > 1.0 || sat[c] < 0.0) {
                if (co->clamp_sat) sat[c] = std::max(std::min(sat[c], 1.0), 0.0);
                else if (sat[c] > 1.001 || sat[c] < -0.001) return 2;
            }
        }
    }
    return 0;
}

}  // extern "C"
