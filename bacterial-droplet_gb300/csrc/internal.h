// internal.h — host-side helpers shared by libttsh's translation units.
#pragma once
#include <string>

namespace ttsh {
// Records `msg` as the calling thread's last error and returns `code`.
int set_error(int code, const std::string& msg);
}  // namespace ttsh
