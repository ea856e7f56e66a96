// The host's waits for a stream, counted and timed (see stream_wait.h).
#include "stream_wait.h"

#include <chrono>

namespace {

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// Polls st until its work is done or limit_ms has passed since t0.
cudaError_t poll_stream(cudaStream_t st, double limit_ms, std::chrono::steady_clock::time_point t0) {
  for (;;) {
    const cudaError_t e = cudaStreamQuery(st);
    if (e != cudaErrorNotReady) return e;
    if (ms_since(t0) >= limit_ms) return cudaErrorTimeout;
  }
}

}  // namespace

cudaError_t flock_stream_wait(cudaStream_t st, WaitStats* w, bool count) {
  if (!w) return cudaStreamSynchronize(st);
  const auto t0 = std::chrono::steady_clock::now();
  cudaError_t e;
  if (w->limit_ms > 0) {
    e = poll_stream(st, w->limit_ms, t0);
    // a query that found the stream busy may leave cudaErrorNotReady as the
    // thread's last error; clear exactly that, so that the launch checks
    // that follow do not report it (any other error stays)
    if (cudaPeekAtLastError() == cudaErrorNotReady) cudaGetLastError();
  } else {
    e = cudaStreamSynchronize(st);
  }
  if (count) {
    w->waits++;
    w->blocked_ms += ms_since(t0);
  }
  return e;
}
