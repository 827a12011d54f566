// sepx_common.h -- error reporting shared by the translation units of the
// library (the message is returned by sepx_last_error()).
#pragma once

namespace sepx {
// records a printf-style message and returns -1
int set_error(const char *fmt, ...);
}  // namespace sepx
