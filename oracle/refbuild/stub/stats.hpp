// Stub of the stats header for building the reference STRUCTURE path only.
// p-value routines are not reached by -structure.
#pragma once
#include <cstdlib>
namespace stats {
template<typename... T> double pchisq(T...) { abort(); }
template<typename... T> double pnorm(T...) { abort(); }
template<typename... T> double pt(T...) { abort(); }
template<typename... T> double pf(T...) { abort(); }
}
