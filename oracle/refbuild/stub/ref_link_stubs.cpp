// Link stubs for building the reference program's STRUCTURE path.
// GWAS (the only translation unit that needs real armadillo) is out of scope:
// its entry point returns without doing anything, as the reference's own
// CalcGWAS does when -gwas is not given.
extern "C" void openblas_set_num_threads(int) {}
template<typename REAL> void CalcGWAS() {}
template void CalcGWAS<double>();
template void CalcGWAS<float>();
