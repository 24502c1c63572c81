// std::map stand-in: same ordered-unique-key semantics (insert keeps the first value).
#pragma once
#include <map>
namespace boost { namespace container { template <class K, class V> using flat_map = std::map<K, V>; } }
