// fused.cu -- the fused FP64 timestep (placeholder until the kernels land).
#include "../../include/flow_gb300.h"
#include "fused.h"

namespace flow {

int fused_solve(Mesh*, int, double*, double*, double*, double*, double*,
                double*, double*, double*, double*, double*, double*, double*,
                double*, double*, double*, double*, double*) {
  return record_error(GB300_ERR_ARG, "fused timestep not available");
}

}  // namespace flow
