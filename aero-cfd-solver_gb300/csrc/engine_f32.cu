// engine_f32.cu -- FP32-bulk / FP64-accumulate instantiation of the device solver.
#include "engine_impl.cuh"

namespace aero {
Engine* make_engine_f32(const std::vector<HostSlots>& hs, const std::vector<aero_case_desc>& cfg,
                        const std::vector<Resolved>& rs, cudaStream_t stream) {
  return new EngineT<float>(hs, cfg, rs, stream);
}
}  // namespace aero
