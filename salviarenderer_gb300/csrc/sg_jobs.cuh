// sg_jobs.cuh -- clears and resolves as jobs of one batched kernel.
#pragma once

#include <cstdint>

#include "sg_common.cuh"

namespace sg {

enum : uint32_t { JOB_FILL = 0, JOB_CLEAR_DS = 1, JOB_RESOLVE = 2 };

struct SurfaceJob {
  uint8_t* dst;
  uint8_t const* src;          // resolve source
  uint64_t n;                  // elements (fill, clear) or pixels (resolve)
  uint32_t kind;
  uint32_t esz;                // element size (fill) / source texel size (resolve)
  uint32_t fmt, dst_fmt;       // depth-stencil format (clear) / source and destination formats (resolve)
  uint32_t samples, flags;
  uint32_t pattern[4];         // converted texel (fill)
  float depth;
  uint32_t stencil;
};

constexpr uint32_t JOBS_PER_LAUNCH = 32;
struct JobList {
  uint32_t n;
  uint32_t count_pass;         // this launch completes its pass: count it in status[1]
  unsigned int* status;        // the device's status words (PassParams::sticky)
  SurfaceJob jobs[JOBS_PER_LAUNCH];
};

}  // namespace sg
