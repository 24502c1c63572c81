#pragma once
#include <random>
namespace boost { namespace random { using std::uniform_real_distribution; } }
