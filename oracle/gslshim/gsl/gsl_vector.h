/* Header-only GSL stand-in: only the opaque type name is referenced by the reference's headers. */
#pragma once
#include <cstddef>
struct gsl_vector;
