// Minimal stand-in for the magic_enum header that the reference code generator
// includes (the reference pins it as a meson wrap at `revision = head`, which is not
// vendored).  Oracle build only: it provides exactly the calls the reference makes
// (enum_integer, enum_count, enum_cast, the enum_range customisation point and the
// bitwise/ostream operator namespaces).  None of them carries code-generation
// arithmetic; enum_count<rv_data_type>() == 6 is pinned by the reference's own
// static_asserts in include/codegen/rv_nodetype.hpp.
#pragma once

#include <cstdint>
#include <optional>
#include <ostream>
#include <string_view>
#include <type_traits>
#include <utility>

namespace magic_enum {
namespace customize {
template <typename E>
struct enum_range {
    static constexpr int min = -128;
    static constexpr int max = 128;
};
}  // namespace customize

namespace detail {
// GCC spells a named enumerator as "E V = scope::name]" and an unnamed value as
// "E V = (scope)7]"; the first character after "V = " tells them apart.
template <typename E, E V>
constexpr bool is_named() {
    constexpr std::string_view sig = __PRETTY_FUNCTION__;
    constexpr auto pos = sig.rfind("V = ");
    static_assert(pos != std::string_view::npos);
    return sig[pos + 4] != '(';
}

template <typename E, int Min, int... I>
constexpr std::size_t count_named(std::integer_sequence<int, I...>) {
    return (std::size_t{0} + ... + (is_named<E, static_cast<E>(Min + I)>() ? 1 : 0));
}

template <typename E, int Min, int... I>
constexpr bool value_named(int v, std::integer_sequence<int, I...>) {
    return ((v == Min + I && is_named<E, static_cast<E>(Min + I)>()) || ...);
}

template <typename E>
constexpr int range_min() {
    using U = std::underlying_type_t<E>;
    constexpr int m = customize::enum_range<E>::min;
    return std::is_unsigned_v<U> && m < 0 ? 0 : m;
}
}  // namespace detail

template <typename E>
constexpr auto enum_integer(E v) noexcept {
    return static_cast<std::underlying_type_t<E>>(v);
}

template <typename E>
constexpr std::size_t enum_count() noexcept {
    constexpr int lo = detail::range_min<E>();
    constexpr int hi = customize::enum_range<E>::max;
    return detail::count_named<E, lo>(std::make_integer_sequence<int, hi - lo + 1>{});
}

template <typename E>
constexpr std::optional<E> enum_cast(int v) noexcept {
    constexpr int lo = detail::range_min<E>();
    constexpr int hi = customize::enum_range<E>::max;
    if (v < lo || v > hi) {
        return std::nullopt;
    }
    if (detail::value_named<E, lo>(v, std::make_integer_sequence<int, hi - lo + 1>{})) {
        return static_cast<E>(v);
    }
    return std::nullopt;
}

template <typename E>
constexpr std::optional<E> enum_cast(unsigned int v) noexcept {
    return enum_cast<E>(static_cast<int>(v));
}

namespace bitwise_operators {
template <typename E, typename = std::enable_if_t<std::is_enum_v<E>>>
constexpr E operator|(E a, E b) noexcept {
    using U = std::underlying_type_t<E>;
    return static_cast<E>(static_cast<U>(a) | static_cast<U>(b));
}
template <typename E, typename = std::enable_if_t<std::is_enum_v<E>>>
constexpr E operator&(E a, E b) noexcept {
    using U = std::underlying_type_t<E>;
    return static_cast<E>(static_cast<U>(a) & static_cast<U>(b));
}
}  // namespace bitwise_operators

namespace ostream_operators {
template <typename E, typename = std::enable_if_t<std::is_enum_v<E>>>
std::ostream& operator<<(std::ostream& os, E v) {
    return os << static_cast<long long>(static_cast<std::underlying_type_t<E>>(v));
}
}  // namespace ostream_operators
}  // namespace magic_enum
