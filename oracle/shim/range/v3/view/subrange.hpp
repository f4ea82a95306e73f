// Stand-in for range-v3's subrange (used by eflib thread_context.h:40).
#pragma once
#include <ranges>
namespace ranges {
using std::ranges::subrange;
}
