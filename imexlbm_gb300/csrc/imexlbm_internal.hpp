// Internal declarations shared by the library's translation units.
#pragma once

#include <cstdint>
#include <string>

namespace imex {

// Record an error for the calling thread (used before a handle exists) and
// return `code`.
int set_thread_error(int code, const std::string& msg);
const char* thread_error();

// The process's test-fault setting (imex_test_set_fault): its kind and value.
int test_fault_kind();
long long test_fault_value();

}  // namespace imex
