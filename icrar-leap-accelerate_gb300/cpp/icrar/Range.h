// icrar::Range (LA/common/Range.h:34-64): a finite linear sequence of indexes.
#pragma once

#include <cstdint>

#include "exception.h"

namespace icrar {

struct Range {
  std::int32_t start;
  std::int32_t interval;
  std::int32_t end;

  Range(int start_, int interval_, int end_) {
    if (start_ < 0) throw icrar::exception("expected a positive integer", __FILE__, __LINE__);
    if (interval_ < 1) throw icrar::exception("expected a positive integer", __FILE__, __LINE__);
    if (end_ < 0) throw icrar::exception("expected a positive integer", __FILE__, __LINE__);
    start = start_;
    interval = interval_;
    end = end_;
  }

  // Number of elements: (end - start) / interval.
  int GetSize() const { return (end - start) / interval; }
};

}  // namespace icrar
