// Work list of the single-kernel momentum assembly (assemble.cu,
// momentum_fused_k). Not part of the C ABI.
//
// The kernel is persistent: its blocks take items from one ticket counter in
// the order of this list. An item is either an edge chunk (kFusedChunk
// consecutive edges: evaluate their coefficients into the edge ring) or a
// row block (kFusedBlock consecutive node rows: sum their incident edges'
// coefficients into CSR values). A row block waits for the edge chunks it
// reads; an edge chunk that reuses a ring slot waits for the row blocks that
// read the slot's previous chunk. Every wait points to items earlier in the
// list, and a block takes a ticket only when it is running, so every item
// waited on is held by a running block: the schedule cannot deadlock,
// whatever the number of resident blocks.
#pragma once

#include <cstdint>
#include <vector>

namespace nw {

constexpr int kFusedChunk = 256;  // edges per edge chunk (one per thread)
constexpr int kFusedBlock = 85;   // node rows per row block (3 threads each)

struct FusedSchedule {
  int64_t chunks = 0;       // edge chunks
  int64_t blocks = 0;       // row blocks
  int64_t ring_chunks = 0;  // ring slots (a power of two); >= chunks: no reuse
  int64_t lag = 0;          // chunks placed between a row block's last input and it
  // items: 2 c for edge chunk c, 2 k + 1 for row block k, in ticket order
  std::vector<int32_t> items;
  // per row block: the range of edge chunks its rows read (lo > hi: none)
  std::vector<int32_t> chunk_lo, chunk_hi;
  // per edge chunk: the range of row blocks that read it (lo > hi: none)
  std::vector<int32_t> block_lo, block_hi;
  // the exact lists the kernel waits on (subsets of the ranges): the
  // distinct chunks each row block reads (CSR: in_ptr, in) and the distinct
  // row blocks reading each chunk (out_ptr, out)
  std::vector<int32_t> in_ptr, in, out_ptr, out;
};

// Builds the schedule for node rows 0..rows-1 whose incidence lists are
// inc[inc_ptr[r] .. inc_ptr[r+1]) (entries edge << 1 | side, bit 31 a flag).
// concurrency: blocks the kernel keeps resident (sets the lag). The ring is
// the smallest power of two of chunks, at most max_ring_chunks, that
// schedules every row block at least `lag` chunks after its last input;
// when none does, it falls back to one slot per chunk (no reuse).
void build_fused_schedule(int64_t num_edges, int64_t rows, const int32_t* inc_ptr,
                          const uint32_t* inc, int64_t concurrency, int64_t max_ring_chunks,
                          FusedSchedule& out);

}  // namespace nw
