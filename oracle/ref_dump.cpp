// Runs the reference program's own grid Fock build and SCF loop and writes
// what they compute to .npy files.
//
// TEST INFRASTRUCTURE (oracle only).  Linked against the reference's
// unmodified translation units (atomicgrid, moleculargrid, gridpoint, cgf,
// functionals, spherical_harmonics, cspline, quadrature, molecule, settings,
// integrals, gamma, dft) and the Eigen/Boost API subset under oracle/shim, by
// oracle/Makefile (`make refdump`).  The members of DFT are private, so the
// reference headers are included with private/protected opened up after every
// standard and shim header has been read; the class layouts are unchanged.
//
//   ref_dump INPUT OUTDIR build P.bin [amp]   one build at a fixed P
//   ref_dump INPUT OUTDIR scf MAXIT TOL       the SCF loop from the core guess
//
// INPUT is a reference input file (settings header, "system:" block); the
// working directory must hold ../basis/<name>.dat, as for the reference's own
// program (molecule.cpp:147-152).  P.bin holds nbf*nbf doubles, column-major.
//
// build: DFT(INPUT) (dft.cpp:30-76: grid, matrices, core-guess density, first
// J), then the steps of one SCF iteration after the eigen-solve at the given
// P: MolecularGrid::set_density + correct_densities (dft.cpp:361-365),
// calculate_electronic_repulsion_matrix (dft.cpp:377-386),
// calculate_exchange_correlation_matrix (dft.cpp:394-433) and calculate_energy
// (dft.cpp:441-447), each timed with std::chrono.
// scf: DFT(INPUT), then iterations of dft.cpp:96-103 until |dE| <= TOL after at
// least three iterations (dft.cpp:95, with TOL in place of 1e-4) or MAXIT.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <map>
#include <regex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>
#include <filesystem>
#include <Eigen/Dense>
#include <boost/format.hpp>
#include <boost/lexical_cast.hpp>
#include <boost/algorithm/string.hpp>
#include <boost/regex.hpp>
#include <boost/filesystem.hpp>
#include <boost/math/special_functions/factorials.hpp>
#include <png.h>

#define private public
#define protected public
#include "dft.h"
#undef private
#undef protected

// declared by the reference (functionals.h:33) but never defined there
Functional::Functional() {}

namespace {

void write_npy(const std::string &path, const std::vector<double> &v, const std::vector<size_t> &shape)
{
    std::string dims;
    for (size_t i = 0; i < shape.size(); ++i) dims += std::to_string(shape[i]) + (shape.size() == 1 ? "," : (i + 1 < shape.size() ? ", " : ""));
    std::string hdr = "{'descr': '<f8', 'fortran_order': False, 'shape': (" + dims + "), }";
    const size_t total = 10 + hdr.size() + 1;
    hdr += std::string((64 - total % 64) % 64, ' ') + "\n";
    std::ofstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot write " + path);
    const char magic[8] = {'\x93', 'N', 'U', 'M', 'P', 'Y', 1, 0};
    f.write(magic, 8);
    const unsigned short hl = (unsigned short)hdr.size();
    const unsigned char hlb[2] = {(unsigned char)(hl & 0xff), (unsigned char)(hl >> 8)};
    f.write(reinterpret_cast<const char *>(hlb), 2);
    f.write(hdr.data(), (std::streamsize)hdr.size());
    f.write(reinterpret_cast<const char *>(v.data()), (std::streamsize)(v.size() * sizeof(double)));
}

// row-major dump of an Eigen-shaped matrix: shape (rows, cols)
template <typename M>
void write_matrix(const std::string &dir, const std::string &name, const M &m)
{
    std::vector<double> v((size_t)(m.rows() * m.cols()));
    for (long i = 0; i < (long)m.rows(); ++i)
        for (long j = 0; j < (long)m.cols(); ++j) v[(size_t)(i * m.cols() + j)] = m(i, j);
    write_npy(dir + "/" + name + ".npy", v, {(size_t)m.rows(), (size_t)m.cols()});
}

void write_vector(const std::string &dir, const std::string &name, const std::vector<double> &v)
{
    write_npy(dir + "/" + name + ".npy", v, {v.size()});
}

double ms_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void dump_grid(DFT &dft, const std::string &out, bool amp)
{
    MolecularGrid &mg = *dft.molgrid;
    const VectorXd w = mg.get_weights();
    const VectorXd rho = mg.get_densities();
    std::vector<double> vw(w.data(), w.data() + w.size()), vr(rho.data(), rho.data() + rho.size());
    std::vector<double> becke, pot, pos;
    for (auto &ag : mg.atomic_grids) {
        for (size_t j = 0; j < ag->grid.size(); ++j) {
            becke.push_back(ag->grid[j].get_becke_weight());
            const vec3 &p = ag->grid[j].get_position();
            pos.push_back(p(0));
            pos.push_back(p(1));
            pos.push_back(p(2));
        }
        for (long j = 0; j < (long)ag->V.size(); ++j) pot.push_back(ag->V(j));
    }
    write_vector(out, "weights", vw);
    write_vector(out, "becke", becke);
    write_vector(out, "rho", vr);
    write_vector(out, "potential", pot);
    write_npy(out + "/positions.npy", pos, {pos.size() / 3, 3});
    if (amp) {
        write_matrix(out, "amplitudes", mg.get_amplitudes());
        std::vector<double> rl, ul;
        size_t nr = 0, nlm = 0;
        for (auto &ag : mg.atomic_grids) {
            nr = (size_t)ag->rho_lm.rows();
            nlm = (size_t)ag->rho_lm.cols();
            for (size_t i = 0; i < nr; ++i)
                for (size_t k = 0; k < nlm; ++k) {
                    rl.push_back(ag->rho_lm((long)i, (long)k));
                    ul.push_back(ag->U_lm((long)i, (long)k));
                }
        }
        write_npy(out + "/rho_lm.npy", rl, {mg.atomic_grids.size(), nr, nlm});
        write_npy(out + "/U_lm.npy", ul, {mg.atomic_grids.size(), nr, nlm});
    }
}

void dump_matrices(DFT &dft, const std::string &out)
{
    write_matrix(out, "J", dft.J);
    write_matrix(out, "XC", dft.XC);
    write_matrix(out, "P", dft.P);
    write_matrix(out, "S", dft.S);
    write_matrix(out, "T", dft.T);
    write_matrix(out, "Vnuc", dft.V);
    write_matrix(out, "H", dft.H);
}

std::vector<double> read_doubles(const std::string &path, size_t n)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot read " + path);
    std::vector<double> v(n);
    f.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(n * sizeof(double)));
    if ((size_t)f.gcount() != n * sizeof(double)) throw std::runtime_error("short file " + path);
    return v;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 5) {
        std::cerr << "usage: ref_dump INPUT OUTDIR build P.bin [amp] | scf MAXIT TOL\n";
        return 2;
    }
    const std::string input = argv[1], out = argv[2], mode = argv[3];
    try {
        std::filesystem::create_directories(out);
        auto t0 = std::chrono::steady_clock::now();
        DFT dft(input);
        const double t_setup = ms_since(t0);
        // the reference leaves these pointers empty (dft.h:45-46); the calls below need them
        dft.integrator = std::make_shared<Integrator>();
        dft.functional = std::make_shared<Functional>();
        const unsigned nbf = dft.mol->get_nr_bfs();

        if (mode == "build") {
            const std::vector<double> pv = read_doubles(argv[4], (size_t)nbf * nbf);
            const bool amp = argc > 5 && std::strcmp(argv[5], "amp") == 0;
            MatrixXXd P = MatrixXXd::Zero(nbf, nbf);
            for (unsigned j = 0; j < nbf; ++j)
                for (unsigned i = 0; i < nbf; ++i) P(i, j) = pv[(size_t)j * nbf + i];
            dft.P = P;
            auto t = std::chrono::steady_clock::now();
            dft.molgrid->set_density(dft.P);
            const double t_dens = ms_since(t);
            const double n_before = dft.molgrid->calculate_density();
            t = std::chrono::steady_clock::now();
            dft.molgrid->correct_densities();
            const double t_corr = ms_since(t);
            const double n_after = dft.molgrid->calculate_density();
            t = std::chrono::steady_clock::now();
            dft.calculate_electronic_repulsion_matrix();
            const double t_hart = ms_since(t);
            t = std::chrono::steady_clock::now();
            dft.calculate_exchange_correlation_matrix();
            const double t_xc = ms_since(t);
            t = std::chrono::steady_clock::now();
            dft.calculate_energy();
            const double t_en = ms_since(t);
            dump_grid(dft, out, amp);
            dump_matrices(dft, out);
            write_vector(out, "scalars", {dft.exc, dft.electronic_repulsion, dft.single_electron_energy, dft.enuc,
                                          dft.et, n_before, n_after});
            write_vector(out, "timings_ms", {t_dens, t_corr, t_hart, t_xc, t_en, t_setup});
        } else if (mode == "scf") {
            const int maxit = std::atoi(argv[4]);
            const double tol = argc > 5 ? std::atof(argv[5]) : 1e-4;
            // the constructor's energy E_0 reads exc before anything sets it
            // (dft.h:68, dft.cpp:441-447); take E_0 with E_xc = 0
            dft.exc = 0.0;
            dft.calculate_energy();
            std::vector<double> hist;
            double old = dft.et;
            for (int it = 1; it <= maxit; ++it) {
                dft.calculate_density_matrix();
                dft.calculate_electronic_repulsion_matrix();
                dft.calculate_exchange_correlation_matrix();
                dft.calculate_energy();
                const double n = dft.molgrid->calculate_density();
                hist.insert(hist.end(), {dft.et, dft.single_electron_energy, dft.electronic_repulsion, dft.exc, n});
                const double diff = std::fabs(dft.et - old);
                old = dft.et;
                if (diff <= tol && it >= 3) break;
            }
            write_npy(out + "/history.npy", hist, {hist.size() / 5, 5});
            dump_grid(dft, out, false);
            dump_matrices(dft, out);
            write_vector(out, "scalars", {dft.exc, dft.electronic_repulsion, dft.single_electron_energy, dft.enuc,
                                          dft.et, dft.molgrid->calculate_density(), 0.0});
        } else {
            std::cerr << "unknown mode " << mode << "\n";
            return 2;
        }
    } catch (const std::exception &e) {
        std::cerr << "ref_dump: " << e.what() << "\n";
        return 1;
    }
    return 0;
}
