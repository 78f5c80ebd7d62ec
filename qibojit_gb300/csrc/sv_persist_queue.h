// sv_persist_queue.h -- the work queue of the persistent batch executor, kept free of
// CUDA types so host code and CPU tests can build and check it.
//
// Every pass of every group becomes one queue entry (a "launch" of the kernel's
// ticket stream): round r holds every group's pass r, groups in the order given
// (largest states first).  An entry owns `ncirc << (tshift - cshift)` consecutive
// tickets from `first`, a ticket being 2^cshift tiles of one circuit, circuits in
// order; it counts finished tiles per circuit at counter offset `cnt` and, from its
// second pass on, waits on the previous pass's counters at `prev` (-1: no wait).
// Every entry's predecessor comes earlier in the queue, so all tickets a ticket waits
// for precede it.
#pragma once

#include <stdint.h>

#include <algorithm>
#include <vector>

namespace sv {

constexpr int kPersistChunkBits = 2;  // up to 4 tiles of one circuit per ticket

struct PersistGroup {
  int npasses;  // passes of the group's plan
  int ncirc;    // circuits in the group
  int tshift;   // log2 tiles per circuit and pass
};

struct PersistEntry {
  int group, pass;
  int64_t first;  // first ticket
  int64_t ntickets;
  int tshift, cshift;
  int cnt, prev;  // counter offsets (prev = -1: a group's first pass)
};

// the queue; *ncounters receives the number of per-circuit counters it uses
inline std::vector<PersistEntry> persist_queue(const std::vector<PersistGroup>& groups, int* ncounters) {
  std::vector<PersistEntry> q;
  std::vector<int> prev(groups.size(), -1);
  int maxp = 0;
  for (const PersistGroup& g : groups) maxp = std::max(maxp, g.npasses);
  int64_t tickets = 0;
  int counters = 0;
  for (int r = 0; r < maxp; r++)
    for (size_t gi = 0; gi < groups.size(); gi++) {
      const PersistGroup& g = groups[gi];
      if (r >= g.npasses) continue;
      PersistEntry e;
      e.group = (int)gi;
      e.pass = r;
      e.first = tickets;
      e.tshift = g.tshift;
      e.cshift = std::min(g.tshift, kPersistChunkBits);
      e.ntickets = (int64_t)g.ncirc << (e.tshift - e.cshift);
      e.cnt = counters;
      e.prev = prev[gi];
      prev[gi] = counters;
      counters += g.ncirc;
      tickets += e.ntickets;
      q.push_back(e);
    }
  if (ncounters) *ncounters = counters;
  return q;
}

}  // namespace sv
