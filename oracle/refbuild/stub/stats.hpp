// Stub of the stats header for building the reference STRUCTURE path only.
// p-value routines are not reached by -structure.
#pragma once
#include <cstdlib>
namespace stats {
// reached by the HWE p-value that the locus diversity filter computes for
// every locus; no output pinned against the reference uses it (no -f_pval),
// so it is a quiet NaN rather than an abort
template<typename... T> double pchisq(T...) { return __builtin_nan(""); }
template<typename... T> double pnorm(T...) { abort(); }
template<typename... T> double pt(T...) { abort(); }
template<typename... T> double pf(T...) { abort(); }
}
