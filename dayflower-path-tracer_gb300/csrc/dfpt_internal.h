// dfpt_internal.h - declarations shared by the host translation units of the renderer core.
#pragma once

#include <stdint.h>

#define FLT_MAX_F 3.402823466e+38f

// Records `code` and a printf-style message as the thread's last error and returns `code`.
int dfpt_fail(int code, const char* fmt, ...);
