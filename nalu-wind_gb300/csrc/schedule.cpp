// Work list of the single-kernel momentum assembly (see schedule.h).
#include "schedule.h"

#include <algorithm>
#include <climits>

namespace nw {

namespace {

// Places the items for ring size S and lag L. Row blocks go in ascending
// order, each once every chunk up to the last one any block so far reads is
// placed and L more chunks have followed. An edge chunk that reuses a slot
// goes once every row block reading the slot's previous chunk was placed,
// also L chunks ago: with about 2 L items in flight, a wait then finds its
// items done. With `relax` (the fallback) the lags are dropped where the
// next item would otherwise be held. False: S too small.
bool place(int64_t nch, int64_t nrb, int64_t S, int64_t L, bool relax,
           const std::vector<int32_t>& cmono, const std::vector<int32_t>& kmono,
           std::vector<int32_t>& items) {
  items.clear();
  items.reserve(size_t(nch + nrb));
  std::vector<int64_t> placed_at(size_t(nrb), 0);  // chunks placed before each row block
  int64_t c = 0, k = 0;
  auto put_row = [&]() {
    placed_at[k] = c;
    items.push_back(int32_t(2 * k++ + 1));
  };
  while (c < nch || k < nrb) {
    while (k < nrb && (c == nch || cmono[k] + L < c)) put_row();
    if (c == nch) continue;
    const int32_t last = c < S ? -1 : kmono[c - S];  // last reader of the slot's chunk
    if (last < k && (last < 0 || placed_at[last] + L <= c || relax)) {
      items.push_back(int32_t(2 * c++));
    } else if (relax && k < nrb && cmono[k] < c) {
      put_row();
    } else {
      return false;
    }
  }
  return true;
}

}  // namespace

void build_fused_schedule(int64_t num_edges, int64_t rows, const int32_t* inc_ptr,
                          const uint32_t* inc, int64_t concurrency, int64_t max_ring_chunks,
                          FusedSchedule& out) {
  FusedSchedule s;
  s.chunks = (num_edges + kFusedChunk - 1) / kFusedChunk;
  s.blocks = (rows + kFusedBlock - 1) / kFusedBlock;
  s.chunk_lo.assign(size_t(s.blocks), INT32_MAX);
  s.chunk_hi.assign(size_t(s.blocks), -1);
  s.block_lo.assign(size_t(s.chunks), INT32_MAX);
  s.block_hi.assign(size_t(s.chunks), -1);
  for (int64_t r = 0; r < rows; ++r) {
    const int32_t k = int32_t(r / kFusedBlock);
    for (int32_t q = inc_ptr[r]; q < inc_ptr[r + 1]; ++q) {
      const int64_t e = (inc[q] & 0x7fffffffu) >> 1;
      const int32_t c = int32_t(e / kFusedChunk);
      s.chunk_lo[k] = std::min(s.chunk_lo[k], c);
      s.chunk_hi[k] = std::max(s.chunk_hi[k], c);
      s.block_lo[c] = std::min(s.block_lo[c], k);
      s.block_hi[c] = std::max(s.block_hi[c], k);
    }
  }
  // distinct (block, chunk) pairs, sorted both ways
  {
    std::vector<int64_t> pairs;
    for (int64_t r = 0; r < rows; ++r)
      for (int32_t q = inc_ptr[r]; q < inc_ptr[r + 1]; ++q)
        pairs.push_back((r / kFusedBlock) << 32 | (((inc[q] & 0x7fffffffu) >> 1) / kFusedChunk));
    std::sort(pairs.begin(), pairs.end());
    pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
    s.in_ptr.assign(size_t(s.blocks) + 1, 0);
    s.out_ptr.assign(size_t(s.chunks) + 1, 0);
    for (int64_t p : pairs) {
      ++s.in_ptr[(p >> 32) + 1];
      ++s.out_ptr[(p & 0xffffffff) + 1];
    }
    for (int64_t k = 0; k < s.blocks; ++k) s.in_ptr[k + 1] += s.in_ptr[k];
    for (int64_t c = 0; c < s.chunks; ++c) s.out_ptr[c + 1] += s.out_ptr[c];
    s.in.resize(pairs.size());
    s.out.resize(pairs.size());
    std::vector<int32_t> pos(s.out_ptr.begin(), s.out_ptr.end() - 1);
    for (size_t i = 0; i < pairs.size(); ++i) {
      s.in[i] = int32_t(pairs[i] & 0xffffffff);  // block-major order
      s.out[pos[pairs[i] & 0xffffffff]++] = int32_t(pairs[i] >> 32);
    }
  }
  // running maxima: the last chunk read by blocks 0..k, the last block
  // reading chunks 0..c
  std::vector<int32_t> cmono(size_t(s.blocks)), kmono(size_t(s.chunks));
  int32_t m = -1;
  for (int64_t k = 0; k < s.blocks; ++k) cmono[k] = m = std::max(m, s.chunk_hi[k]);
  m = -1;
  for (int64_t c = 0; c < s.chunks; ++c) kmono[c] = m = std::max(m, s.block_hi[c]);
  s.lag = std::max<int64_t>(1, concurrency);
  bool done = false;
  for (int64_t S = 64; S < s.chunks && S <= max_ring_chunks; S *= 2) {
    if (place(s.chunks, s.blocks, S, s.lag, false, cmono, kmono, s.items)) {
      s.ring_chunks = S;
      done = true;
      break;
    }
  }
  if (!done) {
    // one slot per chunk: no chunk waits for a slot
    s.ring_chunks = s.chunks;
    place(s.chunks, s.blocks, s.chunks, s.lag, true, cmono, kmono, s.items);
  }
  out = std::move(s);
}

}  // namespace nw
