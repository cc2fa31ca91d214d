// ctx.hpp -- the opaque aero_ctx of the C ABI (shared by the C-ABI translation units).
#pragma once

#include "../../include/aero_gb300.h"
#include "engine.hpp"

#include <cuda_runtime.h>

#include <memory>
#include <string>

struct aero_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  aero_case_desc cfg{};
  std::unique_ptr<aero::Engine> engine;
  std::string error;
};
