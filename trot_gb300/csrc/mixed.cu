// Mixed-precision (tensor-core) path.
#include "mixed.h"

namespace trot {

size_t mixed_workspace_size(const trot_system*, int) { return 0; }

static int not_yet() {
  set_error("mixed precision path not available in this build");
  return TROT_ERR_UNSUPPORTED;
}
int mixed_force_bias(const trot_system*, const Spins&, const double2*, double2*, Carver&, cudaStream_t) { return not_yet(); }
int mixed_local_energy(const trot_system*, const Spins&, const double2*, const double2*, double2*, Carver&,
                       cudaStream_t) { return not_yet(); }
int mixed_apply_trotter(const trot_system*, const Spins&, const double2*, const TrotterArgs&, Carver&, cudaStream_t) {
  return not_yet();
}
int mixed_prop_step(const trot_system*, const Spins&, const trot_state*, const double*, double2*, StepBuffers&,
                    Carver&, cudaStream_t) { return not_yet(); }
}  // namespace trot
