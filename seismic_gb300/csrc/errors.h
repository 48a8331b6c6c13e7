// errors.h -- per-thread message of the last failed call that has no engine
// (seis_create, seis_forward_noalloc); read through seis_last_error(NULL).
#pragma once
#include <string>

namespace seis {
void set_thread_error(const std::string& msg);
}  // namespace seis
