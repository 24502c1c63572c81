// std stand-in for the one boost container alias the reference headers use.
#pragma once
#include <array>
namespace boost { template <class T, std::size_t N> using array = std::array<T, N>; }
