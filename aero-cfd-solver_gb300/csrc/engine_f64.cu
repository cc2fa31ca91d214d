// engine_f64.cu -- plain FP64 instantiation of the device solver.
#include "engine_impl.cuh"

namespace aero {
Engine* make_engine_f64(const std::vector<HostSlots>& hs, const std::vector<aero_case_desc>& cfg,
                        const std::vector<Resolved>& rs, cudaStream_t stream) {
  return new EngineT<double>(hs, cfg, rs, stream);
}
}  // namespace aero
