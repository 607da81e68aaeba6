// FP32-bulk instances of the pass kernels and their launchers.
#include "vk_engine.cuh"

namespace vk {
template struct Engine<float>;
}  // namespace vk
