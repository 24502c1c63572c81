// std::vector stand-in (small_vector only changes allocation, not contents).
#pragma once
#include <vector>
namespace boost { namespace container { template <class T, std::size_t N> using small_vector = std::vector<T>; } }
