// Empty stand-in: with GCC the reference's byte-swap helpers use __builtin_bswap*
// (src/tree.hpp:47-81), so no Boost.Endian symbol is needed by the oracle build.
#pragma once
#include <iterator>
