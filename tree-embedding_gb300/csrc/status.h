// Internal error plumbing shared by every translation unit of libtsvd_gb300.
#pragma once
#include <cstdarg>
#include <cstdio>
#include "../../include/tsvd.h"

namespace tsvd {

// Records a printf-style message for tsvd_last_error() and returns `s`.
tsvd_status fail(tsvd_status s, const char *fmt, ...);

}  // namespace tsvd

#define TSVD_TRY(expr)                    \
  do {                                    \
    tsvd_status _st = (expr);             \
    if (_st != TSVD_OK) return _st;       \
  } while (0)
