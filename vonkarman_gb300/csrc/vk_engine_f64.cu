// FP64 instances of the pass kernels and their launchers.
#include "vk_engine.cuh"

namespace vk {
template struct Engine<double>;
}  // namespace vk
