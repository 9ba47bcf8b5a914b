// The C ABI's thread-local diagnostic (mmr_last_error_message), for entry points
// implemented outside capi.cpp.
#pragma once

#include <stdint.h>

#include <string>

namespace mmr {

// Sets the calling thread's last diagnostic (cleared, without allocating, on success).
void set_last_error(int32_t status, const char *message);

}  // namespace mmr
