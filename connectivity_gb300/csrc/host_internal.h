// Internal host-side helpers shared by the translation units of libgbconn.
#pragma once
#include <cstdint>
#include "gen_common.h"

// Records the detail of a failure for gb_last_error (thread-local).
// `fmt` has one %s, filled with `detail`.
void gb_set_error(const char* fmt, const char* detail);

// R-MAT probabilities as 32-bit fixed-point thresholds.
gb_rmat_thr gb_rmat_thresholds(double a, double b, double c);
