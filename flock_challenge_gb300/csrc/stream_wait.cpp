// The host's waits for a stream, counted and timed (see stream_wait.h).
#include "stream_wait.h"

#include <chrono>

cudaError_t flock_stream_wait(cudaStream_t st, WaitStats* w) {
  if (!w) return cudaStreamSynchronize(st);
  const auto t0 = std::chrono::steady_clock::now();
  const cudaError_t e = cudaStreamSynchronize(st);
  w->waits++;
  w->blocked_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return e;
}
