// The solver template instantiated for the mixed form (FP32 fields and transforms).
#include "solver_impl.cuh"

namespace lesgo {
SolverBase* make_solver_fp32(const Derived& d, int capacity) { return new Solver<float>(d, capacity); }
}  // namespace lesgo
