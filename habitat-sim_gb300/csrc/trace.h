// NVTX ranges around the host-side stages of the renderer (import, draw,
// readback, post-processing, keyframe application) so that a profiler's
// timeline shows where a step's host time goes.  NVTX v3 is header-only:
// without an attached tool a push or pop is a check of one pointer.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace gbr {

class TraceRange {
 public:
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace gbr
