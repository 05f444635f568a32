// Internal declarations shared by the code generator and the runtime of libhyk.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "hyk.h"

namespace hyk {

// A validated copy of a hyk_decomp_t.
struct Dec {
    uint32_t n_eq = 0, n_ops = 0, n_pars = 0;
    std::vector<hyk_uop_t> ops;
    std::vector<hyk_arg_t> rhs;
    std::vector<hyk_event_t> ev;  // events: non-terminal and terminal, in one list
    uint32_t n_u() const { return n_eq + n_ops; }
};

bool load_dec(const hyk_decomp_t *d, Dec &out, std::string &err);

// Result of code generation for one (decomposition, order, arithmetic, block) tuple.
struct GenOut {
    std::string src;          // complete NVRTC translation unit
    uint32_t n_slot = 0;      // shared-memory doubles per lane
    uint32_t par_slot = 0;    // first parameter slot
    uint32_t n_cold = 0;      // cold state rows (orders 1..p in the module's global buffer)
    double flops = 0;         // algorithmic FP64 flops per step per lane
};

// Shared-memory slots per lane for a decomposition at a given order (the
// block size does not change it).
// cold_rows: the layout with cold state rows (their orders 1..p in a global
// buffer, only order 0 in shared memory); *n_cold receives their number.
// split: the recurrences as one function per order (the global-memory lane
// form; implied for the adjoint and for large systems), which keeps the
// reciprocals of order-0 denominators in slots of their own.
uint32_t count_slots(const Dec &d, uint32_t order, bool adjoint = false, bool pin = false, bool cold_rows = false,
                     uint32_t *n_cold = nullptr, bool split = false);

// adjoint: also emit the reverse sweep hyk_jets_bw() and the adjoint kernel
// (and keep every history up to order p-1 for it).
// gmem_stride != 0: Taylor coefficients in a global-memory buffer with that
// slot stride (the number of threads of the fixed grid) instead of shared memory.
// cold_stride != 0: the cold-state-row layout, the global rows with that slot
// stride (the number of threads of the fixed grid).
bool generate(const Dec &d, uint32_t order, bool pin_arith, uint32_t blk, size_t kparams_size, GenOut &out,
              std::string &err, bool adjoint = false, uint64_t gmem_stride = 0, bool high_acc = false,
              bool f32 = false, uint64_t cold_stride = 0, bool split = false);

// Team form (several threads per trajectory): slot count and the share of
// busy threads over the rounds of one order for teams of 1, 2, 4, ..., 32.
struct TeamInfo {
    uint32_t n_slot = 0;       // doubles per trajectory (padded)
    uint32_t n_slot_cold = 0;  // the same with cold state rows (0: the system has none)
    double util[6] = {0, 0, 0, 0, 0, 0};
};
// false (with the reason) when an operation has no team-form code.
bool team_layout(const Dec &d, uint32_t order, TeamInfo &info, std::string &err);
bool generate_team(const Dec &d, uint32_t order, uint32_t team, uint32_t tpb, size_t kparams_size, GenOut &out,
                   std::string &err, bool high_acc = false, bool f32 = false, bool gmem = false, bool cold = false);

// Host (CPU) translation unit of the same recurrences, for checks of the
// generator (team: the team form's recurrences, run by a team of one; cold:
// with cold state rows where the system allows them).
bool generate_host(const Dec &d, uint32_t order, bool adjoint, std::string &src, std::string &err, bool team = false,
                   bool f32 = false, bool cold = false);

// The recurrences in the reference's arithmetic over an element type chosen
// by the includer (a vector of lanes for the compiled CPU stepper).
bool generate_host_batch(const Dec &d, uint32_t order, std::string &src, std::string &err);

}  // namespace hyk
