// extern "C" harness over the reference's dependency-free translation units
// (quadrature.{h,cpp}, cspline.{h,cpp}, gamma.{h,cpp}), compiled from the
// reference sources by oracle/Makefile.  Test infrastructure: used only to pin
// the oracle's Lebedev table, cubic spline and Boys function.
#include "quadrature.h"
#include "cspline.h"
#include "gamma.h"
#include <vector>

extern "C" {

int ref_lebedev_total() { return (int)Quadrature::num_lebedev_coefficients; }

void ref_lebedev(double* out)
{
    for (unsigned i = 0; i < Quadrature::num_lebedev_coefficients; ++i)
        for (int k = 0; k < 4; ++k) out[4 * i + k] = Quadrature::lebedev_coefficients[i][k];
}

void ref_spline_eval(int n, const double* x, const double* y, int nq, const double* xq, double* out)
{
    Cspline s;
    s.set_values(std::vector<double>(x, x + n), std::vector<double>(y, y + n));
    s.generate_spline();
    for (int i = 0; i < nq; ++i) out[i] = s.eval(xq[i]);
}

double ref_fgamma(int m, double x)
{
    GammaInc g;
    return g.Fgamma((double)m, x);
}

}
