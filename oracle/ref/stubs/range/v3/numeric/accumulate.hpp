// Oracle build only: see range/v3/view/zip.hpp.
#pragma once
#include <utility>
namespace ranges {
template <typename R, typename T>
T accumulate(R&& r, T init) {
    for (auto&& v : r) { init = init + v; }
    return init;
}
}  // namespace ranges
