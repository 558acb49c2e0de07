// spx_parse.hh -- host-side parsing of reference DataContainer blobs into ProblemDesc.
#pragma once

#include <cstddef>
#include <cstdint>

#include "spx_params.hh"

namespace spx {

// Parse one plugin blob into pd. slot >= 0 replaces the slot-th boundary (of the parsed
// boundary's class) or distribution instead of appending. Returns an SPX_* code.
int parse_plugin(ProblemDesc& pd, int traj, int role, int kind, const uint8_t* blob, size_t len, int slot);

// Whether trajectory type traj can run on background class bg_kind (the guiding-centre types need
// static fields).
bool background_allowed(int traj, int bg_kind);

// The reference's readiness check plus action-index validation. Returns an SPX_* code.
int check_ready(const ProblemDesc& pd, int traj);

}  // namespace spx
