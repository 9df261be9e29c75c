/* Forced-include prelude for compiling the reference CPU fitter with g++ on
 * Linux (the reference targets MSVC). Test-only: the resulting library is the
 * checker for the oracle restatement, never a product path.
 *
 * - All standard headers come first, so the MSVC-style max/min macros that the
 *   reference's definitions.h defines cannot break later standard includes.
 * - CPUgaussLib.cpp defines its own float erf/erfc; they are renamed so that
 *   they do not collide with the C++ standard library overloads. Nothing on the
 *   B-spline path calls them.
 * - With BSFIT_REF_PROMOTE_DOUBLE the whole fitter is compiled with float
 *   promoted to double: the FP64 oracle of the reference method. */
#ifndef BSFIT_REF_PRELUDE_H
#define BSFIT_REF_PRELUDE_H
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <cmath>
#include <cstring>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <limits>
using std::isnan;
#define erf ref_erf
#define erfc ref_erfc
#ifdef BSFIT_REF_PROMOTE_DOUBLE
#define float double
#endif
#endif
