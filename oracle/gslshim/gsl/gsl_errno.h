/* Header-only GSL stand-in: the reference's Math/Exceptions.h needs GSL_SUCCESS and gsl_strerror. */
#pragma once
#define GSL_SUCCESS 0
inline const char* gsl_strerror(int) { return "gsl stand-in"; }
