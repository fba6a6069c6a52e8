// Oracle build only: stand-in for fmt (the reference pins fmt 8.1.1 as a meson wrap).
// fmt::print is used only by the reference's debug dump, never on the compile path.
#pragma once
#include <ostream>
namespace fmt {
template <typename... Args>
void print(std::ostream&, const char*, Args&&...) {}
}  // namespace fmt
