// The solver template instantiated for the plain FP64 form.
#include "solver_impl.cuh"

namespace lesgo {
SolverBase* make_solver_fp64(const Derived& d, int capacity) { return new Solver<double>(d, capacity); }
}  // namespace lesgo
