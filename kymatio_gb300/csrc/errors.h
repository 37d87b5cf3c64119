// Thread-local text of the last failure inside the library (kym_last_error).
#pragma once

namespace kym {
void set_error_message(const char* where, const char* what);
void clear_error_message();
}  // namespace kym
