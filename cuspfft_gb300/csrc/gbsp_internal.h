// gbsp_internal.h -- helpers shared by the library's translation units.
#pragma once
#include <string>

namespace gbsp {

// Records `msg` as the calling thread's last error and returns `status`.
int set_error(int status, const std::string& msg);

// Smallest 3-smooth (policy 3) or 7-smooth (policy 7) integer >= n.
long next_smooth(long n, int policy);

}  // namespace gbsp
