// pa_error.h -- last-error message of handle-less C ABI calls (per thread).
#pragma once

#include <string>

namespace pa {
inline thread_local std::string g_last_error;
}  // namespace pa
