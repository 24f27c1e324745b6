// tilequeue.cuh -- the asynchronous tile work queue of the persistent
// relaxation kernels (the pit fill's floods and the flat-surface BFS).
//
// Tiles are processed as soon as they are queued, by whichever warp is free:
// no grid-wide pass barriers.  Both users run monotone relaxations (values
// only fall), so the order of the updates does not change their limit; what
// must not happen is two warps processing one tile at once (a slower warp's
// write-back could undo a faster one's lower values).  Each tile therefore
// has a state: idle, queued, processing, processing and queued again
// meanwhile (re-queued when its processing ends), or done (never queued
// again).  `pending` counts tiles that are queued or processing; the queue
// is drained when it reaches 0.  The ring (cap slots, -1 = empty) holds each
// queued tile once, so cap = 2 * tiles + the tickets warps may hold ahead of
// the pushes (kRingSlack > warps in flight) never overflows.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace cageo {

enum : int { kIdle = 0, kQueued = 1, kBusy = 2, kBusyQueued = 3, kDone = 4 };
constexpr int kEmptySlot = -1;
constexpr int kRingSlack = 8192;

struct TileQueue {
  int* state;              // per tile
  int* ring;               // cap slots
  unsigned int cap;
  unsigned int* head;      // tickets handed out (own 128-byte line)
  unsigned int* tail;      // entries pushed (own line)
  unsigned int* pending;   // tiles queued or being processed (own line)
  int* err;                // set to 3 when a state change keeps failing
};

__device__ __forceinline__ void tq_push(const TileQueue& q, int t) {
  const unsigned int pos = atomicAdd(q.tail, 1u);
  // A plain store: the taker swaps the slot for "empty" and retries while
  // it reads empty.
  ((volatile int*)q.ring)[pos % q.cap] = t;
}

// Queue tile t unless it is queued already or done: idle -> queued,
// processing -> processing and queued again.  A single compare-and-swap
// when the state is the one expected.
__device__ __forceinline__ void tq_enqueue(const TileQueue& q, int t) {
  int expect = kIdle;
  for (int it = 0; it < 256; it++) {
    const int old = atomicCAS(&q.state[t], expect, expect == kIdle ? kQueued : kBusyQueued);
    if (old == expect) {
      if (expect == kIdle) {
        atomicAdd(q.pending, 1u);
        tq_push(q, t);
      }
      return;
    }
    if (old != kIdle && old != kBusy) return;  // queued already, or done
    expect = old;
  }
  atomicCAS(q.err, 0, 3);
}

// Lane 0: take the next queued tile.  A warp takes a ticket (the next ring
// position) when the ring looks non-empty and keeps it until the slot is
// filled -- possibly by a later push -- so no claim ever fails.  Returns
// the tile, or -1 while waiting; *ticket carries the ticket between calls
// (-1: none).
__device__ __forceinline__ int tq_try_dequeue(const TileQueue& q, long long* ticket) {
  if (*ticket < 0) {
    if (*(volatile unsigned int*)q.head >= *(volatile unsigned int*)q.tail) return -1;
    *ticket = atomicAdd(q.head, 1u);
  }
  const int t = atomicExch(&q.ring[(unsigned int)*ticket % q.cap], kEmptySlot);
  if (t == kEmptySlot) return -1;
  *ticket = -1;
  // Queued -> processing: only the taker changes a queued tile's state.
  // The fence puts the change before the staging loads, so a neighbour
  // that writes the halo later sees "processing" and queues the tile again.
  ((volatile int*)q.state)[t] = kBusy;
  __threadfence();
  return t;
}

// Lane 0, after the tile's write-back: idle again (done if nothing more can
// change it), or queued again if a neighbour queued it while it was
// processed.
__device__ __forceinline__ void tq_finish(const TileQueue& q, int t, bool done) {
  if (atomicCAS(&q.state[t], kBusy, done ? kDone : kIdle) == kBusy) {
    atomicSub(q.pending, 1u);
  } else if (done) {  // processing and queued again: only the owner changes that state
    ((volatile int*)q.state)[t] = kDone;
    atomicSub(q.pending, 1u);
  } else {
    ((volatile int*)q.state)[t] = kQueued;
    tq_push(q, t);
  }
}

}  // namespace cageo
