// Shared error state of the C ABI (dg_last_error).
#pragma once
#include <string>

namespace dg {
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
}  // namespace dg
