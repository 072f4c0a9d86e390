// Error reporting shared by the library's translation units: every C entry
// point returns a QH_* status and leaves its message for the calling thread,
// read back with qh_last_error().
#pragma once

#include <string>

namespace qhg {

// Record `msg` as the calling thread's last error and return `code`.
int set_error(int code, const std::string& msg);

}  // namespace qhg
