// Shim for folly::fbvector: a std::vector whose first growth reserves room
// for 4096 elements.  The reference keeps pointers into a vector across an
// emplace_back on the same vector (GeneratePredicateEvaluationPlan,
// learner/CandidateLiteralEvaluator.cpp:239-247); with plain std::vector
// growth that reads freed memory once the vector reallocates.  Reserving up
// front keeps every checker run below the first reallocation point (the plans
// built in tests have far fewer than 4096 nodes).
#pragma once
// folly/FBVector.h pulls these in transitively; the reference relies on it.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <memory>
#include <utility>
#include <vector>

#include "folly/Range.h"

namespace folly {
template <class T, class Allocator = std::allocator<T>>
class fbvector : public std::vector<T, Allocator> {
  using Base = std::vector<T, Allocator>;

 public:
  using Base::Base;
  fbvector() = default;
  fbvector(const Base& b) : Base(b) {}
  fbvector(Base&& b) : Base(std::move(b)) {}

  template <class... Args>
  void emplace_back(Args&&... args) {
    grow();
    Base::emplace_back(std::forward<Args>(args)...);
  }
  void push_back(const T& v) {
    grow();
    Base::push_back(v);
  }
  void push_back(T&& v) {
    grow();
    Base::push_back(std::move(v));
  }

 private:
  void grow() {
    if (this->size() == this->capacity())
      this->reserve(std::max<std::size_t>(4096, 2 * this->capacity()));
  }
};
}  // namespace folly
