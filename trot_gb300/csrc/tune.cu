// Process-wide tuning knobs read by the launchers (set by trot_gb300.autotune
// after timing the candidates on the caller's workload).  0 = built-in default.
#include "kernels.h"

namespace trot {
static int g_knobs[TROT_TUNE_COUNT] = {0};
int tune_get(int knob) { return (knob >= 0 && knob < TROT_TUNE_COUNT) ? g_knobs[knob] : 0; }
}  // namespace trot

using namespace trot;

extern "C" {

int trot_set_tuning(int knob, int value) {
  if (knob < 0 || knob >= TROT_TUNE_COUNT) { set_error("unknown tuning knob %d", knob); return TROT_ERR_BAD_SHAPE; }
  if (value < 0 || value > 4096) { set_error("tuning value %d out of range", value); return TROT_ERR_BAD_SHAPE; }
  g_knobs[knob] = value;
  return TROT_OK;
}

int trot_get_tuning(int knob) { return tune_get(knob); }

}  // extern "C"
