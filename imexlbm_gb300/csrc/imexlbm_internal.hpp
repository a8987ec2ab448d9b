// Internal declarations shared by the library's translation units.
#pragma once

#include <cstdint>
#include <string>

namespace imex {

// Record an error for the calling thread (used before a handle exists) and
// return `code`.
int set_thread_error(int code, const std::string& msg);
const char* thread_error();

}  // namespace imex
