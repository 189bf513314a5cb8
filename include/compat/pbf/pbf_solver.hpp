// compat/pbf/pbf_solver.hpp -- forwarding header for code written against the
// reference solver's include path.  With -I include/compat (and -I include),
// a file that says #include "pbf/pbf_solver.hpp" (as the reference's
// benchmark/pbf_benchmark.cu and test/test_pbf_solver.cu do) builds unchanged
// against the C++ shim and links libpbf103.so.
#ifndef PBF103_COMPAT_PBF_SOLVER_HPP
#define PBF103_COMPAT_PBF_SOLVER_HPP
#include "pbf103/pbf_solver.hpp"
#endif
