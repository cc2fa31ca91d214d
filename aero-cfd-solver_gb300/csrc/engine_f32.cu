// engine_f32.cu -- FP32-bulk / FP64-accumulate instantiation of the device solver.
#include "engine_impl.cuh"

namespace aero {
Engine* make_engine_f32(const HostSlots& hs, const aero_case_desc& cfg, const Resolved& rs,
                        cudaStream_t stream) {
  return new EngineT<float>(hs, cfg, rs, stream);
}
}  // namespace aero
