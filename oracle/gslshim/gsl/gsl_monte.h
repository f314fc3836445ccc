/* Header-only GSL stand-in: the reference's Integrate.h declares a function taking this struct. */
#pragma once
#include <cstddef>
struct gsl_monte_function { double (*f)(double*, size_t, void*); size_t dim; void* params; };
