// Self-check of the bounded device waits (see vg_selfcheck.cu).
#pragma once

#include "vg_ctx.h"

namespace vg {

// which 0: a look-back status wait; 1: an mbarrier wait.  Raises
// VG_ERR_TIMEOUT when the wait gave up as it must.
void selfcheck_bounded_wait(Ctx& ctx, int which);

}  // namespace vg
