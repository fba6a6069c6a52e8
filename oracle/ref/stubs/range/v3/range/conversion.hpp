// Oracle build only: see range/v3/view/zip.hpp.
#pragma once
#include <vector>
#include <type_traits>
namespace ranges {
struct to_vector_tag {};
inline constexpr to_vector_tag to_vector{};
template <typename R>
auto operator|(R&& r, to_vector_tag) {
    using V = std::remove_cvref_t<decltype(*std::begin(r))>;
    std::vector<V> out;
    for (auto&& v : r) { out.push_back(v); }
    return out;
}
}  // namespace ranges
