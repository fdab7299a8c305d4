// The per-lane scratch layout of a plan, shared by the launch code (abi.cu)
// and the code generator (codegen.cpp), which bakes its offsets into the
// generated functions.
#pragma once

#include <cstdint>

#include "device.cuh"
#include "symbolic.h"

namespace fo {

inline ScratchLayout layout_of(const HostTables& t) {
  ScratchLayout s;
  int64_t o = 0;
  s.lu = o; o += (int64_t)t.lu_col.size();
  s.negj = o; o += (int64_t)t.j_col.size();
  s.d = o; o += (int64_t)t.R * t.P;
  s.r = o; o += t.R;
  s.y = o; o += t.n;
  s.ynew = o; o += t.n;
  s.f0 = o; o += t.n;
  s.ft = o; o += t.n;
  s.yr = o; o += t.n;
  s.k = o; o += 4LL * t.n;
  s.xs = o; o += t.n;
  s.items = o;
  return s;
}

}  // namespace fo
