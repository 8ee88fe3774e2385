// icrar::Slice (LA/common/Slice.h:36-55, Slice.cc:28-63): a linear sequence
// with -1 wildcards resolved against a collection size by Evaluate.
#pragma once

#include <cstdint>
#include <string>

#include "Range.h"
#include "exception.h"

namespace icrar {

struct Slice {
  std::int32_t start = 0;
  std::int32_t interval = -1;
  std::int32_t end = -1;

  Slice() = default;
  explicit Slice(int interval_) : Slice(0, interval_, -1) {}
  Slice(int start_, int end_) : Slice(start_, end_ == -1 ? -1 : end_ - start_, end_) {}
  Slice(int start_, int interval_, int end_) {
    if (start_ < 0) throw icrar::exception("expected a positive integer", __FILE__, __LINE__);
    if (interval_ < -1) throw icrar::exception("expected a positive integer or -1", __FILE__, __LINE__);
    if (interval_ == 0) throw icrar::exception("expected a non zero integer", __FILE__, __LINE__);
    if (end_ < -1) throw icrar::exception("expected a positive integer or -1", __FILE__, __LINE__);
    if (end_ != -1 && start_ >= end_) throw icrar::exception("range start must be greater than end", __FILE__, __LINE__);
    if (end_ != -1) {
      if (interval_ == -1) interval_ = end_ - start_;
      if (interval_ > (end_ - start_)) throw icrar::exception("range increment out of bounds", __FILE__, __LINE__);
    }
    start = start_;
    interval = interval_;
    end = end_;
  }

  Range Evaluate(int collectionSize) const {
    return Range(start == -1 ? collectionSize : start, interval == -1 ? collectionSize : interval,
                 end == -1 ? collectionSize : end);
  }
};

// Parses the JSON forms the reference accepts for solution intervals:
// an integer interval, or an array [start, interval, end] / [start, end].
Slice ParseSlice(const std::string& json);

}  // namespace icrar
