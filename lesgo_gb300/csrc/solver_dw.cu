// The solver template instantiated for FP64 fields with double-word transforms.
#include "solver_impl.cuh"

namespace lesgo {
SolverBase* make_solver_dw(const Derived& d, int capacity) { return new Solver<double, df64>(d, capacity); }
}  // namespace lesgo
