// Internal declarations shared by the dpg host and device translation units.
#pragma once

#include "dpg.h"

#include <stdint.h>

#include <string>

namespace dpg {

// Records a thread-local error message and returns the status (so `return set_error(...)` works).
dpg_status set_error(dpg_status s, const std::string& msg);

}  // namespace dpg
