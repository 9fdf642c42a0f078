// ORACLE — test infrastructure only.
//
// CPU restatement of Quiqbox.jl v0.6.3's Hartree–Fock driver
// (src/HartreeFock.jl) on a stored ERI tensor, used only by the tests and the
// CPU baseline as the checker.  Restated: symmetric orthogonalisation (:39-42),
// solveFockMatrix with sign stabilisation (:46-56), getD/getGcore/getF/getE
// (:296-350), getCDFE (:392-403), the CoreH / GWH / SAD / Direct initial
// guesses (:195-293) with breakCoeffSymmetry (:71-140), and runHartreeFockCore
// (:1049-1228) with the DD (:1245-1270) and DIIS / EDIIS / ADIIS cores
// (:1273-1394) including subspace reset/eviction.  The DIIS coefficient problem
// is solved by the solver each method names (constraintSolver!, :1479-1487):
// L-BFGS-B (the default, LBFGSBsolver! :1416-1430) or the spectral projected
// gradient (SPGBsolver! :1432-1443), both restated in oracle_diis.cpp, or the
// Lagrange-multiplier solver CMsolver! (:1445-1477) restated here.  The
// coefficient vector of each method persists between its steps, as the
// reference's `cs` does: the solution of one step, with a 1 appended for the
// newest entry, starts the next solve.
//
// LAPACK's `eigen(Hermitian)` is replaced by a cyclic Jacobi eigensolver
// (ascending eigenvalues), LU with partial pivoting replaces `\` and `det`.
// The convergence bookkeeping mirrors the reference run with printInfo=true
// (the mode its tests use), where ΔD and the DIIS error are recorded at every
// step.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <numeric>
#include <functional>

extern "C" {
void qbo_one_body(int kind, int nfun, const int* fp, const double* cen, const int* ijk,
                  const double* alpha, const double* w, int nnuc, const double* Z,
                  const double* R, double* out);
void qbo_eri_tensor(int nfun, const int* fp, const double* cen, const int* ijk,
                    const double* alpha, const double* w, double* eri);
int qbo_diis_solve_iter(int solver, int convex, int n, const double* v, const double* B, double* c);
}

namespace {

using Mat = std::vector<double>;   // n x n, column-major
constexpr double kAtolVal = 4e-16;

struct Dense {
    int n;
    Mat zeros() const { return Mat(size_t(n) * n, 0.0); }
    double& at(Mat& A, int i, int j) const { return A[i + size_t(n) * j]; }
    double at(const Mat& A, int i, int j) const { return A[i + size_t(n) * j]; }
    Mat mul(const Mat& A, const Mat& B) const {   // A*B
        Mat C = zeros();
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < n; ++k) {
                const double b = B[k + size_t(n) * j];
                if (b == 0.0) continue;
                for (int i = 0; i < n; ++i) C[i + size_t(n) * j] += A[i + size_t(n) * k] * b;
            }
        return C;
    }
    Mat tr(const Mat& A) const {
        Mat T = zeros();
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) T[j + size_t(n) * i] = A[i + size_t(n) * j];
        return T;
    }
    Mat add(const Mat& A, const Mat& B, double s = 1.0) const {
        Mat C(A.size());
        for (size_t x = 0; x < A.size(); ++x) C[x] = A[x] + s * B[x];
        return C;
    }
    Mat scale(const Mat& A, double s) const {
        Mat C(A.size());
        for (size_t x = 0; x < A.size(); ++x) C[x] = s * A[x];
        return C;
    }
};

double dotv(const Mat& A, const Mat& B) {
    double s = 0.0;
    for (size_t x = 0; x < A.size(); ++x) s += A[x] * B[x];
    return s;
}

double rms(const Mat& A) {   // rmsOf (Tools.jl:588-589)
    return std::sqrt(dotv(A, A)) / std::sqrt(double(A.size()));
}

// Cyclic Jacobi eigensolver for a symmetric matrix: ascending eigenvalues w,
// orthonormal eigenvectors as columns of V.
void eigh(int n, Mat A, std::vector<double>& w, Mat& V) {
    V.assign(size_t(n) * n, 0.0);
    for (int i = 0; i < n; ++i) V[i + size_t(n) * i] = 1.0;
    auto a = [&](int i, int j) -> double& { return A[i + size_t(n) * j]; };
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) {
                tot += a(i, j) * a(i, j);
                if (i != j) off += a(i, j) * a(i, j);
            }
        if (off <= 1e-30 * tot || off == 0.0) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = a(p, q);
                if (std::fabs(apq) < 1e-300) continue;
                const double theta = (a(q, q) - a(p, p)) / (2 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) /
                                 (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {   // columns p, q
                    const double akp = a(k, p), akq = a(k, q);
                    a(k, p) = c * akp - s * akq;
                    a(k, q) = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {   // rows p, q
                    const double apk = a(p, k), aqk = a(q, k);
                    a(p, k) = c * apk - s * aqk;
                    a(q, k) = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = V[k + size_t(n) * p], vkq = V[k + size_t(n) * q];
                    V[k + size_t(n) * p] = c * vkp - s * vkq;
                    V[k + size_t(n) * q] = s * vkp + c * vkq;
                }
            }
    }
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::vector<double> d(n);
    for (int i = 0; i < n; ++i) d[i] = a(i, i);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return d[x] < d[y]; });
    Mat Vs(size_t(n) * n);
    w.resize(n);
    for (int j = 0; j < n; ++j) {
        w[j] = d[order[j]];
        std::memcpy(&Vs[size_t(n) * j], &V[size_t(n) * order[j]], sizeof(double) * n);
    }
    V.swap(Vs);
}

// LU with partial pivoting: solves A x = b in place; returns det(A)
double lu_solve(int n, std::vector<double> A, std::vector<double>& b) {
    double det = 1.0;
    std::vector<int> piv(n);
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int i = k + 1; i < n; ++i)
            if (std::fabs(A[i + size_t(n) * k]) > std::fabs(A[p + size_t(n) * k])) p = i;
        if (A[p + size_t(n) * k] == 0.0) return 0.0;
        if (p != k) {
            for (int j = 0; j < n; ++j) std::swap(A[k + size_t(n) * j], A[p + size_t(n) * j]);
            std::swap(b[k], b[p]);
            det = -det;
        }
        const double piv_v = A[k + size_t(n) * k];
        det *= piv_v;
        for (int i = k + 1; i < n; ++i) {
            const double f = A[i + size_t(n) * k] / piv_v;
            A[i + size_t(n) * k] = f;
            for (int j = k + 1; j < n; ++j) A[i + size_t(n) * j] -= f * A[k + size_t(n) * j];
            b[i] -= f * b[k];
        }
    }
    for (int i = n - 1; i >= 0; --i) {
        double s = b[i];
        for (int j = i + 1; j < n; ++j) s -= A[i + size_t(n) * j] * b[j];
        b[i] = s / A[i + size_t(n) * i];
    }
    return det;
}

double lu_det(int n, const std::vector<double>& A) {
    std::vector<double> b(n, 0.0);
    return lu_solve(n, A, b);
}

struct System {
    int n;
    Dense M;
    Mat S, H, X;
    const double* eri;   // n^4 column-major
    int nspin;           // 1 RHF, 2 UHF
    int N[2];
};

// getOrthonormalization(:Symmetric) (HartreeFock.jl:39-42)
Mat orthonormalization(const Dense& M, const Mat& S) {
    std::vector<double> s;
    Mat U;
    eigh(M.n, S, s, U);
    Mat X = M.zeros();
    for (int k = 0; k < M.n; ++k) {
        const double f = 1.0 / std::sqrt(s[k]);
        for (int j = 0; j < M.n; ++j)
            for (int i = 0; i < M.n; ++i)
                X[i + size_t(M.n) * j] += U[i + size_t(M.n) * k] * f * U[j + size_t(M.n) * k];
    }
    return X;
}

// solveFockMatrix (HartreeFock.jl:46-56)
Mat solve_fock(const Dense& M, const Mat& X, const Mat& F, std::vector<double>* evals = nullptr) {
    Mat Fp = M.mul(M.tr(X), M.mul(F, X));
    for (int j = 0; j < M.n; ++j)   // Hermitian(.) takes the upper triangle
        for (int i = j + 1; i < M.n; ++i) Fp[i + size_t(M.n) * j] = Fp[j + size_t(M.n) * i];
    std::vector<double> e;
    Mat Cx;
    eigh(M.n, Fp, e, Cx);
    Mat C = M.mul(X, Cx);
    for (int j = 0; j < M.n; ++j)
        if (C[size_t(M.n) * j] < 0)
            for (int i = 0; i < M.n; ++i) C[i + size_t(M.n) * j] = -C[i + size_t(M.n) * j];
    if (evals) *evals = e;
    return C;
}

// getD (HartreeFock.jl:296-299)
Mat density(const Dense& M, const Mat& C, int nocc) {
    Mat D = M.zeros();
    for (int k = 0; k < nocc; ++k)
        for (int j = 0; j < M.n; ++j) {
            const double cj = C[j + size_t(M.n) * k];
            for (int i = 0; i < M.n; ++i) D[i + size_t(M.n) * j] += C[i + size_t(M.n) * k] * cj;
        }
    return D;
}

// getGcore (HartreeFock.jl:305-319): G_μν = Σ DJ_λσ (μν|λσ) − Σ DK_λσ (μλ|σν)
Mat gcore(const System& s, const Mat& DJ, const Mat& DK) {
    const int64_t n = s.n;
    Mat G(size_t(n) * n);
    for (int64_t nu = 0; nu < n; ++nu)
        for (int64_t mu = 0; mu <= nu; ++mu) {
            double r = 0.0;
            for (int64_t sg = 0; sg < n; ++sg)
                for (int64_t la = 0; la < n; ++la) {
                    r += DJ[la + n * sg] * s.eri[mu + n * (nu + n * (la + n * sg))];
                    r -= DK[la + n * sg] * s.eri[mu + n * (la + n * (sg + n * nu))];
                }
            G[mu + n * nu] = r;
            G[nu + n * mu] = r;
        }
    return G;
}

// getG + getF (HartreeFock.jl:322-335)
std::vector<Mat> fock(const System& s, const std::vector<Mat>& D) {
    std::vector<Mat> F;
    if (D.size() == 1) {
        F.push_back(s.M.add(s.H, gcore(s, s.M.scale(D[0], 2.0), D[0])));
    } else {
        const Mat Dt = s.M.add(D[0], D[1]);
        F.push_back(s.M.add(s.H, gcore(s, Dt, D[0])));
        F.push_back(s.M.add(s.H, gcore(s, Dt, D[1])));
    }
    return F;
}

// getE (HartreeFock.jl:339-342)
double energy(const System& s, const Mat& F, const Mat& D) {
    return dotv(D, s.M.add(s.H, F)) / 2;
}

// get2SpinQuantity (HartreeFock.jl:344): RHF doubles the single sector
Mat two_spin(const System& s, const std::vector<Mat>& D) {
    return D.size() == 1 ? s.M.scale(D[0], 2.0) : s.M.add(D[0], D[1]);
}
double two_spin(const std::vector<double>& E) { return E.size() == 1 ? 2 * E[0] : E[0] + E[1]; }

struct Step {
    std::vector<Mat> C, D, F;
    std::vector<double> E;
    Mat Dtot;
    double Etot;
};

// getCDFE (HartreeFock.jl:392-403)
Step cdfe(const System& s, const std::vector<Mat>& F) {
    Step r;
    for (int k = 0; k < s.nspin; ++k) {
        r.C.push_back(solve_fock(s.M, s.X, F[k]));
        r.D.push_back(density(s.M, r.C[k], s.N[k]));
    }
    r.F = fock(s, r.D);
    for (int k = 0; k < s.nspin; ++k) r.E.push_back(energy(s, r.F[k], r.D[k]));
    r.Dtot = two_spin(s, r.D);
    r.Etot = two_spin(r.E);
    return r;
}

// breakCoeffSymmetryCore (HartreeFock.jl:71-101)
std::vector<Mat> break_symmetry_core(const Dense& M, const Mat& X, const Mat& C1, const Mat& C2) {
    const int n = M.n;
    // inv(Hermitian(X)): X = S^{-1/2} is symmetric positive definite
    std::vector<double> e;
    Mat U;
    Mat Xs = X;
    for (int j = 0; j < n; ++j)
        for (int i = j + 1; i < n; ++i) Xs[i + size_t(n) * j] = Xs[j + size_t(n) * i];
    eigh(n, Xs, e, U);
    Mat inv = M.zeros();
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i)
                inv[i + size_t(n) * j] += U[i + size_t(n) * k] * U[j + size_t(n) * k] / e[k];
    Mat o1 = M.mul(inv, C1), o2 = M.mul(inv, C2);
    for (int j = 0; j < n; ++j) {
        Mat& O = (j % 2 == 0) ? o1 : o2;   // counter odd -> first sector
        double* col = &O[size_t(n) * j];
        int idx = 0;
        double mag = std::fabs(col[0]);
        for (int i = 1; i < n; ++i)
            if (std::fabs(col[i]) > mag) { mag = std::fabs(col[i]); idx = i; }
        const double val = col[idx];
        if (std::fabs(mag - 1.0) < std::sqrt(2.220446049250313e-16)) {
            col[idx] *= -val;
        } else {
            col[idx] = 0.0;
            double nrm = 0.0;
            for (int i = 0; i < n; ++i) nrm += col[i] * col[i];
            nrm = std::sqrt(nrm);
            for (int i = 0; i < n; ++i) col[i] /= nrm;
        }
    }
    return {M.mul(X, o1), M.mul(X, o2)};
}

// CMsolver! (HartreeFock.jl:1445-1477) on the (m+1)-bordered system
void cm_solver(bool convex, std::vector<double>& c, const std::vector<double>& v,
               std::vector<double> B) {
    const int m = int(v.size());
    const double pert = 1000 * kAtolVal;
    auto getA = [&](const std::vector<double>& Bm) {
        std::vector<double> A(size_t(m + 1) * (m + 1), 0.0);
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < m; ++i) A[i + size_t(m + 1) * j] = Bm[i + size_t(m) * j];
        for (int i = 0; i < m; ++i) {
            A[i + size_t(m + 1) * m] = 1.0;
            A[m + size_t(m + 1) * i] = 1.0;
        }
        return A;
    };
    std::vector<double> b(m + 1);
    for (int i = 0; i < m; ++i) b[i] = -v[i];
    b[m] = 1.0;
    for (int guard = 0; guard < 100000; ++guard) {
        std::vector<double> A = getA(B);
        while (lu_det(m + 1, A) == 0.0) {
            for (int i = 0; i < m; ++i) B[i + size_t(m) * i] += pert;
            A = getA(B);
        }
        std::vector<double> x = b;
        lu_solve(m + 1, A, x);
        c.assign(x.begin(), x.begin() + m);
        const bool neg = std::any_of(c.begin(), c.end(), [](double t) { return t < 0; });
        if (!convex || !neg) return;
        // powerset(sortperm(abs.(c)), 1): subsets by size, combinations in order
        std::vector<int> perm(m);
        std::iota(perm.begin(), perm.end(), 0);
        std::stable_sort(perm.begin(), perm.end(),
                         [&](int p, int q) { return std::fabs(c[p]) < std::fabs(c[q]); });
        for (int sz = 1; sz <= m; ++sz) {
            std::vector<int> comb(sz);
            std::iota(comb.begin(), comb.end(), 0);
            while (true) {
                std::vector<char> drop(m + 1, 0);
                for (int t : comb) drop[perm[t]] = 1;
                std::vector<int> keep;
                for (int i = 0; i <= m; ++i)
                    if (!drop[i]) keep.push_back(i);
                const int k = int(keep.size());
                std::vector<double> At(size_t(k) * k), bt(k);
                for (int jj = 0; jj < k; ++jj) {
                    bt[jj] = b[keep[jj]];
                    for (int ii = 0; ii < k; ++ii)
                        At[ii + size_t(k) * jj] = A[keep[ii] + size_t(m + 1) * keep[jj]];
                }
                if (lu_det(k, At) != 0.0) {
                    lu_solve(k, At, bt);
                    std::vector<double> cl(m, 0.0);
                    for (int jj = 0; jj < k - 1; ++jj) cl[keep[jj]] = bt[jj];
                    c = cl;
                    if (!std::any_of(c.begin(), c.end(), [](double t) { return t < 0; })) return;
                }
                int pos = sz - 1;   // next combination
                while (pos >= 0 && comb[pos] == m - sz + pos) --pos;
                if (pos < 0) break;
                ++comb[pos];
                for (int t = pos + 1; t < sz; ++t) comb[t] = comb[t - 1] + 1;
            }
        }
        for (int i = 0; i < m; ++i) B[i + size_t(m) * i] += pert;
    }
}

struct Trace {                    // HFtempInfo (HartreeFock.jl:419-436), one per spin
    std::vector<Mat> Cs, Ds, Fs;
    std::vector<double> Es;
};

struct Shared {
    std::vector<Mat> Dtots;
    std::vector<double> Etots;
};

// updateHFtempInfo! (HartreeFock.jl:463-477)
void push_step(size_t maxLen, std::vector<Trace>& t, Shared& sh, const Step& r) {
    for (size_t k = 0; k < t.size(); ++k) {
        auto pushT = [&](std::vector<Mat>& v, const Mat& x) {
            while (v.size() >= maxLen) v.erase(v.begin());
            v.push_back(x);
        };
        pushT(t[k].Cs, r.C[k]);
        pushT(t[k].Ds, r.D[k]);
        pushT(t[k].Fs, r.F[k]);
        t[k].Es.push_back(r.E[k]);
    }
    while (sh.Dtots.size() >= maxLen) sh.Dtots.erase(sh.Dtots.begin());
    sh.Dtots.push_back(r.Dtot);
    sh.Etots.push_back(r.Etot);
}

// popHFtempInfo! (HartreeFock.jl:479-494)
void pop_steps(std::vector<Trace>& t, Shared& sh, int count) {
    for (auto& tv : t)
        for (int c = 0; c < count; ++c) {
            tv.Cs.pop_back(); tv.Ds.pop_back(); tv.Fs.pop_back(); tv.Es.pop_back();
        }
    for (int c = 0; c < count; ++c) { sh.Dtots.pop_back(); sh.Etots.pop_back(); }
}

// getEresidual / getErrorNrms (HartreeFock.jl:1230-1237,1298-1299)
Mat residual(const Dense& M, const Mat& F, const Mat& D, const Mat& S) {
    return M.add(M.mul(F, M.mul(D, S)), M.mul(S, M.mul(D, F)), -1.0);
}
double error_norm(const System& s, const std::vector<Trace>& t) {
    double acc = 0.0;
    for (auto& tv : t) acc += rms(residual(s.M, tv.Fs.back(), tv.Ds.back(), s.S));
    return acc / t.size();
}

double stdev(const std::vector<double>& v) {
    const double m = std::accumulate(v.begin(), v.end(), 0.0) / v.size();
    double s = 0.0;
    for (double x : v) s += (x - m) * (x - m);
    return std::sqrt(s / (v.size() - 1));
}

// isOscillateConverged (Tools.jl:291-315) for the minimum-seeking case
bool oscillate_converged(const std::vector<double>& seq, double tar, int minLen, int maxRemains) {
    const int len = int(seq.size());
    if (len < minLen) return false;   // head returns a single zero -> length < 2
    const int slice = std::min(maxRemains, len / 3 + 1);
    std::vector<double> tail(seq.end() - slice, seq.end());
    if (tail.size() < 2) return false;
    std::sort(tail.begin(), tail.end());
    std::vector<double> valleys(tail.begin(), tail.begin() + (tail.size() / 2 + 1));
    const double target = *std::min_element(valleys.begin(), valleys.end());
    return stdev(valleys) <= 0.8 * tar && std::fabs(target - seq.back()) <= tar;
}

// One SCF method core: DD (HartreeFock.jl:1245-1270) or a DIIS variant (:1335-1394)
struct Core {
    int method;   // 0 DD, 1 DIIS, 2 EDIIS, 3 ADIIS
    int solver = 0;   // 0 L-BFGS-B (default, HartreeFock.jl:17), 1 SPG, 2 Lagrange multipliers
    double damp = 0.75;
    int diis_size = 15;
    double reset = 1000 * kAtolVal;
    std::vector<std::vector<double>> cs;
    std::vector<std::vector<Mat>> Dss, Fss;
    std::vector<std::vector<double>> Ess;
};

Step run_core(const System& s, Core& core, std::vector<Trace>& t) {
    std::vector<Mat> Fn;
    if (core.method == 0) {
        std::vector<Mat> Dn;
        for (int k = 0; k < s.nspin; ++k) {
            const Mat Dnew = density(s.M, solve_fock(s.M, s.X, t[k].Fs.back()), s.N[k]);
            Dn.push_back(s.M.add(s.M.scale(Dnew, 1 - core.damp), s.M.scale(t[k].Ds.back(), core.damp)));
        }
        Fn = fock(s, Dn);
        return cdfe(s, Fn);
    }
    for (int k = 0; k < s.nspin; ++k) {
        auto& Ds = core.Dss[k];
        auto& Fs = core.Fss[k];
        auto& Es = core.Ess[k];
        const int m = int(Ds.size());
        std::vector<double> v(m, 0.0), B(size_t(m) * m, 0.0);
        if (core.method == 1) {          // DIIScore (:1301-1315)
            std::vector<Mat> R;
            for (int i = 0; i < m; ++i)
                R.push_back(s.M.mul(s.M.tr(s.X), s.M.mul(residual(s.M, Fs[i], Ds[i], s.S), s.X)));
            for (int j = 0; j < m; ++j)
                for (int i = 0; i <= j; ++i) B[i + size_t(m) * j] = B[j + size_t(m) * i] = dotv(R[i], R[j]);
        } else if (core.method == 2) {   // EDIIScore (:1273-1285)
            v = Es;
            for (int j = 0; j < m; ++j)
                for (int i = 0; i <= j; ++i)
                    B[i + size_t(m) * j] = B[j + size_t(m) * i] =
                        -dotv(s.M.add(Ds[i], Ds[j], -1.0), s.M.add(Fs[i], Fs[j], -1.0));
        } else {                          // ADIIScore (:1287-1296)
            for (int i = 0; i < m; ++i) v[i] = dotv(s.M.add(Ds[i], Ds[m - 1], -1.0), Fs[m - 1]);
            for (int j = 0; j < m; ++j)
                for (int i = 0; i < m; ++i)
                    B[i + size_t(m) * j] =
                        dotv(s.M.add(Ds[i], Ds[m - 1], -1.0), s.M.add(Fs[j], Fs[m - 1], -1.0));
        }
        if (core.solver == 2)
            cm_solver(core.method != 1, core.cs[k], v, B);
        else
            qbo_diis_solve_iter(core.solver, core.method != 1, m, v.data(), B.data(), core.cs[k].data());
        Mat F = s.M.zeros();
        for (int i = 0; i < m; ++i) F = s.M.add(F, Fs[i], core.cs[k][i]);
        Fn.push_back(F);
    }
    Step r = cdfe(s, Fn);
    for (int k = 0; k < s.nspin; ++k) {
        auto& c = core.cs[k];
        auto& Ds = core.Dss[k];
        auto& Fs = core.Fss[k];
        auto& Es = core.Ess[k];
        c.push_back(1.0);
        Ds.push_back(r.D[k]);
        Fs.push_back(r.F[k]);
        Es.push_back(r.E[k]);
        if (Es.size() > 2 && Es.back() - Es[Es.size() - 2] > core.reset) {
            const size_t keep = Es.size() - 2;   // keepOnly! of the second-to-last
            c = {c[keep]};
            Ds = {Ds[keep]};
            Fs = {Fs[keep]};
            Es = {Es[keep]};
        } else if (int(c.size()) > core.diis_size) {
            const size_t pi = std::max_element(Es.begin(), Es.end()) - Es.begin();
            c.erase(c.begin() + pi);
            Ds.erase(Ds.begin() + pi);
            Fs.erase(Fs.begin() + pi);
            Es.erase(Es.begin() + pi);
        }
    }
    return r;
}

struct Result {
    int converged;
    int steps;
    double E;
};

// runHartreeFockCore (HartreeFock.jl:1049-1228)
Result scf_core(const System& s, std::vector<Mat> C0, int nmeth, const int* methods,
                const double* intervals, const int* solvers, double ratio1, double ratio2, double oscThr,
                int maxStep, bool earlyStop, std::vector<Trace>& t, Shared& sh) {
    // initializeSCF (:526-542)
    t.assign(s.nspin, Trace{});
    std::vector<Mat> D;
    for (int k = 0; k < s.nspin; ++k) D.push_back(density(s.M, C0[k], s.N[k]));
    std::vector<Mat> F = fock(s, D);
    std::vector<double> E;
    for (int k = 0; k < s.nspin; ++k) {
        E.push_back(energy(s, F[k], D[k]));
        t[k].Cs = {C0[k]};
        t[k].Ds = {D[k]};
        t[k].Fs = {F[k]};
        t[k].Es = {E[k]};
    }
    sh.Dtots = {two_spin(s, D)};
    sh.Etots = {two_spin(E)};
    std::vector<double> dEs = {0.0}, dDrms = {0.0}, dFrms = {error_norm(s, t)};
    const int HFminItr = 10, oscSize = 15;
    int converged = 1;
    int i = 0;
    for (int l = 0; l < nmeth; ++l) {
        const bool endM = (l == nmeth - 1);
        const double bp = intervals[l];
        const size_t len = methods[l] == 0 ? 3 : 15;   // max(HFinterMatStoreSizes..., cache size)
        Core core;
        core.method = methods[l];
        core.solver = solvers ? solvers[l] : 0;
        if (core.method != 0) {   // initializeHFcore for DIIS types (:1335-1360)
            const size_t init = std::min<size_t>(core.diis_size, t[0].Ds.size());
            for (int k = 0; k < s.nspin; ++k) {
                std::vector<double> c(init);
                for (size_t x = 0; x < init; ++x) c[x] = double(x + 1);
                core.cs.push_back(c);
                core.Dss.emplace_back(t[k].Ds.end() - init, t[k].Ds.end());
                core.Fss.emplace_back(t[k].Fs.end() - init, t[k].Fs.end());
                core.Ess.emplace_back(t[k].Es.end() - init, t[k].Es.end());
            }
        }
        const double fluc = std::max(10 * bp, 1.5e-3);
        const double dFbp = ratio1 * bp, dDbp = ratio2 * bp;
        const double dEosc = std::max(bp, oscThr), dFosc = ratio1 * dEosc, dDosc = ratio2 * dEosc;
        converged = 0;
        int n = 0;
        while (true) {
            if (!(i < maxStep)) break;
            ++i;
            ++n;
            push_step(len, t, sh, run_core(s, core, t));
            dEs.push_back(sh.Etots.back() - sh.Etots[sh.Etots.size() - 2]);
            dDrms.push_back(rms(s.M.add(sh.Dtots.back(), sh.Dtots[sh.Dtots.size() - 2], -1.0)));
            dFrms.push_back(error_norm(s, t));
            const double dE = dEs.back(), dD = dDrms.back(), dF = dFrms.back(), adE = std::fabs(dE);
            double th0 = bp, th1 = dDbp;
            if (dF > dFbp) { th0 = 0.0; th1 = 0.0; }
            if (adE <= th0 && dD <= th1) { converged = 1; break; }
            if (n > 1 && i > HFminItr && dE > fluc) {
                bool isOsc = false;
                if (oscThr > 0) {
                    isOsc = oscillate_converged(sh.Etots, 10 * dEosc, HFminItr, oscSize);
                    if (isOsc && adE <= dEosc && (endM ? (dF <= dFosc && dD <= dDosc) : true)) {
                        converged = 2;
                        break;
                    }
                }
                if (earlyStop && !isOsc) {
                    bool raising = true;
                    for (int j = 0; j <= HFminItr / 3; ++j)
                        if (!(dEs[dEs.size() - 1 - j] > 10 * fluc)) raising = false;
                    if (raising) {
                        const int memLen = int(t[0].Cs.size());
                        const int rb = std::min(HFminItr / 3 + 1, std::max(memLen - 1, 0));
                        pop_steps(t, sh, rb);
                        i -= rb;
                        break;
                    }
                }
            }
        }
    }
    return Result{converged, i, sh.Etots.back()};
}

}  // namespace

extern "C" {

// Hartree–Fock on a stored ERI tensor.
//   methods: 0 DD, 1 DIIS, 2 EDIIS, 3 ADIIS; solvers (per method, may be null = all
//            L-BFGS-B): 0 L-BFGS-B, 1 SPG, 2 Lagrange multipliers
//   guess:   0 CoreH, 1 GWH, 2 SAD, 3 Direct (C0 given, nspin matrices)
// Outputs (nspin blocks of n*n / n): C, D, F, orbital energies; scalars in info:
//   info[0] = E_elec, info[1] = converged (0 no, 1 yes, 2 oscillation), info[2] = steps
int qbo_hartree_fock(int nfun, const int* fp, const double* cen, const int* ijk,
                     const double* alpha, const double* w, int nnuc, const double* Z,
                     const double* R, int nalpha, int nbeta, int uhf, int guess,
                     const double* C0, int nmeth, const int* methods, const double* intervals,
                     const int* solvers, double ratio1, double ratio2, double oscThr, int maxStep, int earlyStop,
                     double* Cout, double* Dout, double* Fout, double* eps, double* info) {
    const int n = nfun;
    if ((!uhf && nalpha != nbeta) || nmeth < 1) return -1;
    System s;
    s.n = n;
    s.M = Dense{n};
    s.S.resize(size_t(n) * n);
    Mat T(size_t(n) * n), V(size_t(n) * n);
    qbo_one_body(0, n, fp, cen, ijk, alpha, w, 0, nullptr, nullptr, s.S.data());
    qbo_one_body(1, n, fp, cen, ijk, alpha, w, 0, nullptr, nullptr, T.data());
    qbo_one_body(2, n, fp, cen, ijk, alpha, w, nnuc, Z, R, V.data());
    s.H = s.M.add(T, V);   // coreHamiltonian = Summator(kinetic, nuclear) (Samplers.jl:110-121)
    std::vector<double> eri(size_t(n) * n * n * n);
    qbo_eri_tensor(n, fp, cen, ijk, alpha, w, eri.data());
    s.eri = eri.data();
    s.X = orthonormalization(s.M, s.S);
    s.nspin = uhf ? 2 : 1;
    s.N[0] = nalpha;
    s.N[1] = nbeta;

    std::vector<Mat> Cinit;
    if (guess == 3) {
        for (int k = 0; k < s.nspin; ++k) Cinit.emplace_back(C0 + size_t(k) * n * n, C0 + size_t(k + 1) * n * n);
    } else {
        Mat Hg = s.H;
        if (guess == 1) {   // GWH (:235-254)
            for (int j = 0; j < n; ++j)
                for (int i = 0; i <= j; ++i) {
                    const double r = 3 * s.S[i + size_t(n) * j] *
                                     (s.H[i + size_t(n) * i] + s.H[j + size_t(n) * j]) / 8;
                    Hg[i + size_t(n) * j] = r;
                    Hg[j + size_t(n) * i] = r;
                }
        }
        if (guess == 2) {   // SAD (:266-293): per-atom UHF/ADIIS on the atomic core Hamiltonian
            System a = s;
            a.nspin = 2;
            Mat Da = s.M.zeros(), Db = s.M.zeros();
            for (int c = 0; c < nnuc; ++c) {
                Mat Va(size_t(n) * n);
                qbo_one_body(2, n, fp, cen, ijk, alpha, w, 1, Z + c, R + 3 * c, Va.data());
                a.H = s.M.add(T, Va);
                // initializeOrbCoeffData(:CoreH, UHF, matOverlap, atmOneBody): S is passed as X
                const Mat Cg = solve_fock(s.M, s.S, a.H);
                std::vector<Mat> Ca = break_symmetry_core(s.M, s.S, Cg, Cg);
                std::vector<Trace> ta;
                Shared sa;
                const int m3 = 3;
                const double iv = std::max(1e-2, 10 * kAtolVal);
                scf_core(a, Ca, 1, &m3, &iv, nullptr, 1000.0, 1000.0, 5e-6, 50, true, ta, sa);
                Da = s.M.add(Da, ta[0].Ds.back());
                Db = s.M.add(Db, ta[1].Ds.back());
            }
            Da = s.M.scale(Da, 1.0 / nnuc);
            Db = s.M.scale(Db, 1.0 / nnuc);
            if (!uhf) {
                const Mat Dh = s.M.scale(s.M.add(Da, Db), 0.5);
                std::vector<Mat> F = fock(s, {Dh});
                Cinit = {solve_fock(s.M, s.X, F[0])};
            } else {
                std::vector<Mat> F = fock(s, {Da, Db});
                Mat C1 = solve_fock(s.M, s.X, F[0]), C2 = solve_fock(s.M, s.X, F[1]);
                // breakCoeffSymmetry(UHF, X, (C1, C2)) (:108-119)
                std::vector<double> e;
                Mat U, Xs = s.X;
                eigh(n, Xs, e, U);
                Mat inv = s.M.zeros();
                for (int k = 0; k < n; ++k)
                    for (int j = 0; j < n; ++j)
                        for (int i = 0; i < n; ++i)
                            inv[i + size_t(n) * j] += U[i + size_t(n) * k] * U[j + size_t(n) * k] / e[k];
                if (rms(s.M.mul(inv, s.M.add(C1, C2, -1.0))) < 0.1)
                    Cinit = break_symmetry_core(s.M, s.X, C1, C2);
                else
                    Cinit = {C1, C2};
            }
        } else {            // CoreH (:221-226) or GWH
            const Mat C = solve_fock(s.M, s.X, Hg);
            if (uhf) Cinit = break_symmetry_core(s.M, s.X, C, C);
            else Cinit = {C};
        }
    }
    std::vector<Trace> t;
    Shared sh;
    const Result r = scf_core(s, Cinit, nmeth, methods, intervals, solvers, ratio1, ratio2, oscThr, maxStep,
                              earlyStop != 0, t, sh);
    for (int k = 0; k < s.nspin; ++k) {
        std::memcpy(Cout + size_t(k) * n * n, t[k].Cs.back().data(), sizeof(double) * n * n);
        std::memcpy(Dout + size_t(k) * n * n, t[k].Ds.back().data(), sizeof(double) * n * n);
        std::memcpy(Fout + size_t(k) * n * n, t[k].Fs.back().data(), sizeof(double) * n * n);
        std::vector<double> e;
        solve_fock(s.M, s.X, t[k].Fs.back(), &e);   // getOrbitalOccupations (:708-750)
        std::memcpy(eps + size_t(k) * n, e.data(), sizeof(double) * n);
    }
    info[0] = r.E;
    info[1] = r.converged;
    info[2] = r.steps;
    return 0;
}

// CMsolver! (HartreeFock.jl:1445-1477) on its own: c (n) receives the coefficients.
void qbo_diis_cm(int convex, int n, const double* v, const double* B, double* c) {
    std::vector<double> cv(c, c + n), vv(v, v + n), Bv(B, B + size_t(n) * n);
    cm_solver(convex != 0, cv, vv, Bv);
    std::memcpy(c, cv.data(), sizeof(double) * n);
}

// Symmetric eigen-decomposition exposed for tests (ascending).
void qbo_eigh(int n, const double* A, double* w, double* V) {
    std::vector<double> e;
    Mat U;
    eigh(n, Mat(A, A + size_t(n) * n), e, U);
    std::memcpy(w, e.data(), sizeof(double) * n);
    std::memcpy(V, U.data(), sizeof(double) * n * n);
}

}  // extern "C"
