// icrar::ComputeImplementation (LA/core/compute_implementation.h:33-42) with the
// GB300 value added: "gb300" selects the sm_103a implementation of this library.
#pragma once

#include <string>

namespace icrar {

enum class ComputeImplementation {
  cpu,    // reference Eigen implementation (not part of this library)
  cuda,   // reference CUDA implementation (not part of this library)
  gb300,  // GB300-native implementation (sm_103a kernels behind the leap_gb300 C ABI)
};

// true if value was converted (TryParseComputeImplementation, LA/core/compute_implementation.cc:31-56);
// "casa" and "eigen" stay deprecated aliases of cpu.
bool TryParseComputeImplementation(const std::string& value, ComputeImplementation& out);

}  // namespace icrar
