// Internal declarations shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "../../include/flock_gpu.h"

constexpr int FLOCK_K_LOG = 14;
constexpr int FLOCK_K = 1 << FLOCK_K_LOG;

int flock_launch_witness(const flock_compression* d_in, size_t n_in, int n_blocks_log, void* d_z, void* d_a,
                         void* d_b, void* d_stripe, cudaStream_t stream);

// NTT twiddle tables: device copy of the breadth-first table for a domain of
// 2^log_d (layer l at offset 2^l - 1), built on the host once per size.
const void* flock_ntt_twiddles(int log_d);
int flock_launch_ntt(void* d_data, const void* d_src, int log_d, int log_num_ntts, int start_layer,
                     cudaStream_t stream);

int flock_launch_merkle(const void* d_data, size_t n_leaves, size_t leaf_bytes, void* d_tree,
                        cudaStream_t stream);
