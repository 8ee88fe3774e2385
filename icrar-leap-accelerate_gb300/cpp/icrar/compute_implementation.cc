#include "compute_implementation.h"

#include <iostream>

namespace icrar {

bool TryParseComputeImplementation(const std::string& value, ComputeImplementation& out) {
  if (value == "casa" || value == "eigen") {
    std::cerr << "warning: argument '" << value << "' deprecated, use 'cpu' instead\n";
    out = ComputeImplementation::cpu;
    return true;
  }
  if (value == "cpu") {
    out = ComputeImplementation::cpu;
    return true;
  }
  if (value == "cuda") {
    out = ComputeImplementation::cuda;
    return true;
  }
  if (value == "gb300") {
    out = ComputeImplementation::gb300;
    return true;
  }
  return false;
}

}  // namespace icrar
