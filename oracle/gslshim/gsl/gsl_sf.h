/* Header-only GSL stand-in. The KDTree path calls gsl_sf_gamma once, for the kernel
   normalisation Gamma(ND/2+1) (src/KDTree/KDTree.cxx:1158); std::tgamma stands in for it. */
#pragma once
#include <cmath>
inline double gsl_sf_gamma(double x) { return std::tgamma(x); }
