// cm_internal.h -- declarations shared by the host and device translation
// units of libcm (not part of the public ABI).
#pragma once

#include <cstdarg>
#include <cstdint>
#include <string>

#include "../../include/cm.h"

// Records a formatted message for cm_last_error() and returns `code`.
int cm_fail(int code, const char *fmt, ...);
