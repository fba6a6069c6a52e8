// Oracle build only: stand-in for range-v3 0.12.0, used by the reference solely for
// its stage-timing table (rv_generator.cpp), never on the compile path.
#pragma once
#include <tuple>
#include <vector>
#include <cstddef>
#include <algorithm>
namespace ranges { namespace views {
template <typename... R>
auto zip(R&... rs) {
    std::size_t n = std::min({static_cast<std::size_t>(std::size(rs))...});
    std::vector<std::tuple<decltype(*std::begin(rs))...>> out;
    for (std::size_t i = 0; i < n; ++i) {
        out.emplace_back(*(std::begin(rs) + i)...);
    }
    return out;
}
} }  // namespace ranges::views
