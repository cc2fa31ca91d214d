// engine_f64.cu -- plain FP64 instantiation of the device solver.
#include "engine_impl.cuh"

namespace aero {
Engine* make_engine_f64(const HostSlots& hs, const aero_case_desc& cfg, const Resolved& rs,
                        cudaStream_t stream) {
  return new EngineT<double>(hs, cfg, rs, stream);
}
}  // namespace aero
