#pragma once
#include <random>
namespace boost { namespace random { using std::mt19937; using std::mt19937_64; } using std::mt19937; using std::mt19937_64; }
