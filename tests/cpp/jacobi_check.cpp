// Eigen-decomposition check of dftg_host::jacobi_eigh: reads n and an n x n
// column-major symmetric matrix from stdin, prints the eigenvalues and then
// the eigenvectors (column-major), one number per line.
#include <cstdio>
#include <iostream>
#include <vector>

#include "dftg.hpp"

int main()
{
    int n = 0;
    std::cin >> n;
    std::vector<double> A((size_t)n * n);
    for (double &x : A) std::cin >> x;
    std::vector<double> w, V;
    dftg_host::jacobi_eigh(n, A, w, V);
    for (double x : w) std::printf("%.17g\n", x);
    for (double x : V) std::printf("%.17g\n", x);
    return 0;
}
