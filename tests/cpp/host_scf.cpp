// SCF through the C++ host mirror (include/dftg.hpp).  Reads a molecule and
// flattened basis from a text file:
//   natoms nbf nprim
//   Z x y z                       (natoms lines, bohr)
//   atom l m n nprim              (nbf lines)
//   alpha coef                    (nprim lines)
// and prints "E <energy> ITER <n>" plus the energy of every iteration.
// usage: host_scf <molecule file> <radial> <lebedev order> <lmax> <fp64|mixed> <tol> [device]
// With "device" the SCF runs in the device driver (dftg_host::DeviceSCF).
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>

#include "dftg.hpp"

int main(int argc, char **argv)
{
    if (argc < 7) {
        std::fprintf(stderr, "usage: %s mol.txt nrad leb lmax fp64|mixed tol\n", argv[0]);
        return 2;
    }
    std::ifstream in(argv[1]);
    dftg_host::Molecule mol;
    int natoms = 0, nbf = 0, nprim = 0;
    in >> natoms >> nbf >> nprim;
    mol.Z.resize(natoms);
    mol.xyz.resize(3 * (size_t)natoms);
    for (int a = 0; a < natoms; ++a) in >> mol.Z[a] >> mol.xyz[3 * a] >> mol.xyz[3 * a + 1] >> mol.xyz[3 * a + 2];
    mol.bf_atom.resize(nbf);
    mol.bf_lmn.resize(3 * (size_t)nbf);
    mol.bf_nprim.resize(nbf);
    for (int i = 0; i < nbf; ++i)
        in >> mol.bf_atom[i] >> mol.bf_lmn[3 * i] >> mol.bf_lmn[3 * i + 1] >> mol.bf_lmn[3 * i + 2] >> mol.bf_nprim[i];
    mol.alpha.resize(nprim);
    mol.coef.resize(nprim);
    for (int k = 0; k < nprim; ++k) in >> mol.alpha[k] >> mol.coef[k];
    if (!in) {
        std::fprintf(stderr, "bad molecule file\n");
        return 2;
    }
    const int prec = std::string(argv[5]) == "mixed" ? DFTG_PREC_MIXED : DFTG_PREC_FP64;
    try {
        if (argc > 7 && std::string(argv[7]) == "device") {
            dftg_host::DeviceSCF scf(mol, (unsigned)std::atoi(argv[2]), (unsigned)std::atoi(argv[3]),
                                     (unsigned)std::atoi(argv[4]), prec, 0, std::atof(argv[6]));
            const double e = scf.scf();
            const std::vector<double> h = scf.get(DFTG_SCF_HISTORY);
            for (size_t i = 0; i < h.size(); i += DFTG_SCF_HIST_W) std::printf("IT %.15f\n", h[i]);
            std::printf("E %.15f ITER %d NPTS %zu\n", e, scf.iterations(), scf.molgrid().get_grid_size());
            return 0;
        }
        dftg_host::DFT dft(mol, (unsigned)std::atoi(argv[2]), (unsigned)std::atoi(argv[3]), (unsigned)std::atoi(argv[4]),
                           prec);
        const double e = dft.scf(std::atof(argv[6]));
        for (double h : dft.history()) std::printf("IT %.15f\n", h);
        std::printf("E %.15f ITER %zu NPTS %zu\n", e, dft.history().size(), dft.molgrid().get_grid_size());
    } catch (const std::exception &ex) {
        std::fprintf(stderr, "error: %s\n", ex.what());
        return 1;
    }
    return 0;
}
