// Stub of the gcem header for building the reference STRUCTURE path only.
// The incomplete gamma/beta functions are not reached by -structure.
#pragma once
#include <cstdlib>
namespace gcem {
template<typename A, typename B> double incomplete_gamma(A, B) { abort(); }
template<typename A, typename B, typename C> double incomplete_beta(A, B, C) { abort(); }
}
