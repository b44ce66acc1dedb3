// dftg.hpp -- C++ host mirror of DFTCXX's grid call surface over the C ABI.
//
// Header-only (C++17).  Keeps the class names and call order of the
// reference so that its DFT driver can switch to the GB300 build with few
// edits:
//   MolecularGrid  (moleculargrid.h:84-167): set_grid_parameters, create_grid,
//                  set_density, correct_densities, calculate_density,
//                  calculate_hartree_potential, get_weights / get_densities /
//                  get_amplitudes, get_grid_size
//   DFT            (dft.h, dft.cpp:84-142, 184-226, 300-447): one-electron
//                  matrices, canonical orthogonalisation, SCF with the
//                  reference's linear damping, energy
//   DeviceSCF      the same SCF with every step on the GPU (dftg_scf_*): one
//                  CUDA graph launch per SCF
// Matrices are nbf x nbf column-major std::vector<double> (the reference uses
// Eigen's default column-major MatrixXXd).  Errors from the C ABI are thrown
// as std::runtime_error on this side of the boundary only.
#ifndef DFTG_HPP
#define DFTG_HPP

#include <cmath>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "dftg.h"

namespace dftg_host {

inline void check(int rc)
{
    if (rc != DFTG_OK) throw std::runtime_error(std::string("dftg: ") + dftg_last_error());
}

// Atoms and the flattened contracted-Gaussian basis (the dftg_basis layout):
// function i sits on atom bf_atom[i] with powers bf_lmn[3i..3i+2] and
// bf_nprim[i] primitives taken in order from alpha / coef.
struct Molecule {
    std::vector<int> Z;
    std::vector<double> xyz;          // [natoms][3] bohr
    std::vector<int> bf_atom, bf_lmn, bf_nprim;
    std::vector<double> alpha, coef;

    int natoms() const { return (int)Z.size(); }
    int nbf() const { return (int)bf_atom.size(); }
    int nelec() const
    {
        int n = 0;
        for (int z : Z) n += z;
        return n;
    }
};

class MolecularGrid {
public:
    // MolecularGrid(std::shared_ptr<Molecule>) (moleculargrid.cpp:31-34)
    explicit MolecularGrid(const Molecule &mol) : mol_(mol) {}
    MolecularGrid(const MolecularGrid &) = delete;
    MolecularGrid &operator=(const MolecularGrid &) = delete;
    ~MolecularGrid()
    {
        if (ctx_) dftg_destroy(ctx_);
    }

    // moleculargrid.cpp:175-179 (lebedev_order: 0..10 as settings.h:64-78, 11 = 302 points)
    void set_grid_parameters(unsigned radial_points, unsigned lebedev_order, unsigned lmax, int device = 0)
    {
        params_ = dftg_grid_params{(int)radial_points, (int)lebedev_order, (int)lmax, device};
    }

    // moleculargrid.cpp:193-261: points, Becke weights and amplitudes on the device
    void create_grid()
    {
        if (ctx_) dftg_destroy(ctx_);
        ctx_ = nullptr;
        dftg_molecule m{mol_.natoms(), mol_.Z.data(), mol_.xyz.data()};
        dftg_basis b{mol_.nbf(), mol_.bf_atom.data(), mol_.bf_lmn.data(), mol_.bf_nprim.data(), mol_.alpha.data(),
                     mol_.coef.data()};
        check(dftg_create(&m, &b, &params_, &ctx_));
        check(dftg_set_precision(ctx_, precision_));
    }

    // DFTG_PREC_FP64 (default) or DFTG_PREC_MIXED
    void set_precision(int precision)
    {
        precision_ = precision;
        if (ctx_) check(dftg_set_precision(ctx_, precision));
    }

    void set_density(const std::vector<double> &P) { check(dftg_set_density(ctx(), P.data())); }
    double correct_densities()
    {
        double s = 0.0;
        check(dftg_correct_densities(ctx(), &s));
        return s;
    }
    double calculate_density()
    {
        double n = 0.0;
        check(dftg_calculate_density(ctx(), &n));
        return n;
    }
    std::vector<double> calculate_hartree_potential()
    {
        std::vector<double> J(nn());
        check(dftg_calculate_hartree_potential(ctx(), J.data()));
        return J;
    }
    // DFT::calculate_exchange_correlation_matrix (dft.cpp:394-433): (XC, E_xc)
    std::pair<std::vector<double>, double> calculate_xc()
    {
        std::vector<double> XC(nn());
        double exc = 0.0;
        check(dftg_calculate_xc(ctx(), XC.data(), &exc));
        return {XC, exc};
    }

    struct FockParts {
        std::vector<double> J, XC;
        double exc = 0.0, nelec = 0.0, ej = 0.0;
    };
    // the four calls above in one (dft.cpp:361-433), plus E_J = 2 tr(P J) summed on the grid
    FockParts fock_build(const std::vector<double> &P)
    {
        FockParts f;
        f.J.resize(nn());
        f.XC.resize(nn());
        check(dftg_fock_build(ctx(), P.data(), f.J.data(), f.XC.data(), &f.exc, &f.nelec));
        check(dftg_get_energies(ctx(), &f.exc, &f.ej, &f.nelec));
        return f;
    }

    size_t get_grid_size() const
    {
        size_t n = 0;
        check(dftg_grid_size(ctx_, &n));
        return n;
    }
    std::vector<double> get_weights() const { return points(&dftg_get_weights, 1); }
    std::vector<double> get_densities() const { return points(&dftg_get_densities, 1); }
    std::vector<double> get_amplitudes() const { return points(&dftg_get_amplitudes, (size_t)mol_.nbf()); }

    void one_electron(std::vector<double> &S, std::vector<double> &T, std::vector<double> &V)
    {
        S.assign(nn(), 0.0);
        T.assign(nn(), 0.0);
        V.assign(nn(), 0.0);
        check(dftg_one_electron(ctx(), S.data(), T.data(), V.data()));
    }
    double nuclear_repulsion() const
    {
        double e = 0.0;
        check(dftg_nuclear_repulsion(ctx_, &e));
        return e;
    }

    dftg_ctx *ctx() const
    {
        if (!ctx_) throw std::runtime_error("dftg: create_grid() has not been called");
        return ctx_;
    }

private:
    size_t nn() const { return (size_t)mol_.nbf() * (size_t)mol_.nbf(); }
    std::vector<double> points(int (*get)(const dftg_ctx *, double *, size_t), size_t mult) const
    {
        std::vector<double> out(get_grid_size() * mult);
        check(get(ctx(), out.data(), out.size()));
        return out;
    }

    Molecule mol_;
    dftg_grid_params params_{15, 7, 8, 0};   // the "medium" preset, settings.cpp:166-170
    int precision_ = DFTG_PREC_FP64;
    dftg_ctx *ctx_ = nullptr;
};

// Symmetric eigen-decomposition by cyclic Jacobi rotations (A column-major
// n x n, destroyed).  Eigenvalues ascending in w, eigenvectors in the columns of V.
inline void jacobi_eigh(int n, std::vector<double> A, std::vector<double> &w, std::vector<double> &V)
{
    V.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
    auto a = [&](int i, int j) -> double & { return A[(size_t)j * n + i]; };
    auto v = [&](int i, int j) -> double & { return V[(size_t)j * n + i]; };
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, diag = 0.0;
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) (i == j ? diag : off) += a(i, j) * a(i, j);
        if (off <= 1e-30 * diag || off == 0.0) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = a(p, q);
                if (std::fabs(apq) < 1e-300) continue;
                const double theta = (a(q, q) - a(p, p)) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {   // A <- A G (columns p, q)
                    const double akp = a(k, p), akq = a(k, q);
                    a(k, p) = c * akp - s * akq;
                    a(k, q) = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {   // A <- G^T A (rows p, q)
                    const double apk = a(p, k), aqk = a(q, k);
                    a(p, k) = c * apk - s * aqk;
                    a(q, k) = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = v(k, p), vkq = v(k, q);
                    v(k, p) = c * vkp - s * vkq;
                    v(k, q) = s * vkp + c * vkq;
                }
            }
    }
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    for (int i = 1; i < n; ++i)   // insertion sort by eigenvalue
        for (int j = i; j > 0 && a(idx[j], idx[j]) < a(idx[j - 1], idx[j - 1]); --j) std::swap(idx[j], idx[j - 1]);
    std::vector<double> Vs((size_t)n * n);
    w.resize(n);
    for (int j = 0; j < n; ++j) {
        w[j] = a(idx[j], idx[j]);
        for (int i = 0; i < n; ++i) Vs[(size_t)j * n + i] = v(i, idx[j]);
    }
    V.swap(Vs);
}

// C = A B for column-major n x n matrices, with optional transpose of A
inline std::vector<double> matmul(int n, const std::vector<double> &A, const std::vector<double> &B, bool transA = false)
{
    std::vector<double> C((size_t)n * n, 0.0);
    for (int j = 0; j < n; ++j)
        for (int k = 0; k < n; ++k) {
            const double b = B[(size_t)j * n + k];
            if (b == 0.0) continue;
            for (int i = 0; i < n; ++i)
                C[(size_t)j * n + i] += (transA ? A[(size_t)i * n + k] : A[(size_t)k * n + i]) * b;
        }
    return C;
}

// Closed-shell LDA SCF with the reference's iteration (dft.cpp:84-142):
// F = H + 2J + XC, X = U diag(lambda^-1/2), P = C_occ C_occ^T, and
// P <- (1 - alpha) P_new + alpha P_old with alpha = 0.5 after the first density.
class DFT {
public:
    DFT(const Molecule &mol, unsigned radial_points, unsigned lebedev_order, unsigned lmax,
        int precision = DFTG_PREC_FP64, int device = 0)
        : mol_(mol), grid_(mol), n_(mol.nbf())
    {
        grid_.set_grid_parameters(radial_points, lebedev_order, lmax, device);
        grid_.set_precision(precision);
        grid_.create_grid();
        std::vector<double> S, T, V;
        grid_.one_electron(S, T, V);   // DFT::construct_matrices (dft.cpp:184-199)
        H_.resize(S.size());
        for (size_t i = 0; i < S.size(); ++i) H_[i] = T[i] + V[i];
        enuc_ = grid_.nuclear_repulsion();
        std::vector<double> lam, U;
        jacobi_eigh(n_, S, lam, U);    // DFT::calculate_transformation_matrix (dft.cpp:300-316)
        X_.assign((size_t)n_ * n_, 0.0);
        for (int j = 0; j < n_; ++j)
            for (int i = 0; i < n_; ++i) X_[(size_t)j * n_ + i] = U[(size_t)j * n_ + i] / std::sqrt(lam[j]);
        J_.assign((size_t)n_ * n_, 0.0);
        XC_.assign((size_t)n_ * n_, 0.0);
        density_matrix();              // first density from H (dft.cpp:216-226)
        grid_.set_density(P_);
        grid_.correct_densities();
        J_ = grid_.calculate_hartree_potential();
        ej_ = two_trace(P_, J_);
        energy_ = energy();
    }

    double scf(double tol = 1e-4, int max_iter = 100, int min_iter = 3)
    {
        double old = energy_, diff = 1.0;
        int it = 0;
        while (diff > tol || it < min_iter) {
            ++it;
            density_matrix();
            MolecularGrid::FockParts f = grid_.fock_build(P_);
            J_ = std::move(f.J);
            XC_ = std::move(f.XC);
            exc_ = f.exc;
            ej_ = f.ej;                    // 2 tr(P J), summed on the grid in FP64
            energy_ = energy();
            history_.push_back(energy_);
            diff = std::fabs(energy_ - old);
            old = energy_;
            if (it >= max_iter) break;
        }
        return energy_;
    }

    double get_energy() const { return energy_; }
    const std::vector<double> &get_density_matrix() const { return P_; }
    const std::vector<double> &history() const { return history_; }
    MolecularGrid &molgrid() { return grid_; }

private:
    double two_trace(const std::vector<double> &A, const std::vector<double> &B) const
    {
        double s = 0.0;
        for (size_t i = 0; i < A.size(); ++i) s += A[i] * B[i];   // tr(A B) for symmetric A, B
        return 2.0 * s;
    }

    // DFT::calculate_density_matrix (dft.cpp:330-366)
    void density_matrix(double alpha = 0.5)
    {
        std::vector<double> F((size_t)n_ * n_);
        for (size_t i = 0; i < F.size(); ++i) F[i] = H_[i] + 2.0 * J_[i] + XC_[i];
        const std::vector<double> Fp = matmul(n_, X_, matmul(n_, F, X_), true);
        std::vector<double> eps, Cp;
        jacobi_eigh(n_, Fp, eps, Cp);
        const std::vector<double> C = matmul(n_, X_, Cp);
        const int nocc = mol_.nelec() / 2;
        std::vector<double> Pn((size_t)n_ * n_, 0.0);
        for (int j = 0; j < n_; ++j)
            for (int i = 0; i < n_; ++i) {
                double s = 0.0;
                for (int k = 0; k < nocc; ++k) s += C[(size_t)k * n_ + i] * C[(size_t)k * n_ + j];
                Pn[(size_t)j * n_ + i] = s;
            }
        if (P_.empty()) P_ = Pn;
        else
            for (size_t i = 0; i < P_.size(); ++i) P_[i] = (1.0 - alpha) * Pn[i] + alpha * P_[i];
    }

    // DFT::calculate_energy (dft.cpp:441-447)
    double energy() const { return two_trace(P_, H_) + ej_ + enuc_ + exc_; }

    Molecule mol_;
    MolecularGrid grid_;
    int n_;
    std::vector<double> H_, X_, J_, XC_, P_, history_;
    double enuc_ = 0.0, exc_ = 0.0, ej_ = 0.0, energy_ = 0.0;
};

// The reference's SCF (dft.cpp:84-142) run by the device driver: set-up in the
// constructor, scf() iterates to convergence in one CUDA graph launch.
class DeviceSCF {
public:
    DeviceSCF(const Molecule &mol, unsigned radial_points, unsigned lebedev_order, unsigned lmax,
              int precision = DFTG_PREC_FP64, int device = 0, double tol = 1e-4, int max_iter = 100)
        : grid_(mol), n_(mol.nbf())
    {
        grid_.set_grid_parameters(radial_points, lebedev_order, lmax, device);
        grid_.set_precision(precision);
        grid_.create_grid();
        dftg_scf_params p{0, 0.5, tol, 3, max_iter, 0};
        check(dftg_scf_init(grid_.ctx(), &p));
    }

    double scf()
    {
        double e = 0.0;
        check(dftg_scf_run(grid_.ctx(), &e, &iterations_));
        return e;
    }

    int iterations() const { return iterations_; }

    std::vector<double> get(int what) const   // DFTG_SCF_P, _J, _XC, _H, _X, _EPS, _HISTORY
    {
        std::vector<double> out((size_t)n_ * n_ + (size_t)DFTG_SCF_HIST_W * DFTG_SCF_MAX_ITER);
        size_t cnt = 0;
        check(dftg_scf_get(grid_.ctx(), what, out.data(), out.size(), &cnt));
        out.resize(cnt);
        return out;
    }

    MolecularGrid &molgrid() { return grid_; }

private:
    MolecularGrid grid_;
    int n_;
    int iterations_ = 0;
};

}  // namespace dftg_host

#endif  // DFTG_HPP
