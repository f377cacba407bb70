// The scan's hand-off of candidate regions to the host batch engine (plain
// C++, shared by the CUDA translation units and engine.cpp).
#pragma once
#include <cstdint>

#include "saber_gpu.h"

namespace saber {

// The batch engine's candidate regions, capped per query (and triaged) on
// the device: the kept regions in region order (grouped by query) with
// their positions in the capped list, in pinned memory owned by the handle
// (valid until its next scan).
struct RegionSink {
    float lambda = 0.f, logk = 0.f;  // for the triage features
    const saber_region* regs = nullptr;
    const uint32_t* src = nullptr;
    const uint64_t* sbase = nullptr;  // per kept region: its subject's first residue
    const uint32_t* slen = nullptr;   // and length
    uint64_t n = 0;                  // kept regions
    uint64_t ncap = 0;               // regions after the per-query cap
    bool triaged = false;            // a model dropped regions
    bool collecting = false;         // feature rows were collected
};

}  // namespace saber
