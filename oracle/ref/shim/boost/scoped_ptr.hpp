// unique_ptr stand-in for boost::scoped_ptr.
#pragma once
#include <memory>
namespace boost {
template <class T> class scoped_ptr : public std::unique_ptr<T> {
 public:
  explicit scoped_ptr(T* p = nullptr) : std::unique_ptr<T>(p) {}
};
}  // namespace boost
