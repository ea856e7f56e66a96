// The host's waits for a stream, counted and timed, optionally bounded.
//
// A round of the prover ends with the host reading a few bytes the stream
// produced (a round's partial sums, a grind result, a Merkle root): the
// host waits for the stream there. Counting those waits and the host time
// spent blocked in them splits a phase's wall time into the host's own work
// (launch calls, transcript, host rounds) and the time it waits on the GPU.
// (A flag written into mapped host memory by the stream and polled by the
// host measured no faster than cudaStreamSynchronize on a GB300, 8.7 against
// 8.5 us from launch to return, so the unbounded wait is the stream sync.)
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

struct WaitStats {
  uint64_t waits = 0;     // waits so far
  double blocked_ms = 0;  // host time spent in them
  double limit_ms = 0;    // > 0: a wait gives up after this long
};

// Waits until the stream's queued work is done: cudaStreamSynchronize, or,
// with w->limit_ms > 0, polls the stream and returns cudaErrorTimeout once
// the limit has passed (the queued work keeps running; a later wait or sync
// on the stream sees it finish). Counted and timed in *w when `count`;
// w == nullptr: a plain synchronisation.
cudaError_t flock_stream_wait(cudaStream_t st, WaitStats* w, bool count = true);
