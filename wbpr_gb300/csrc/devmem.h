// Device memory of libwbpr (CUDA translation units only).
//
// Graphs and batches take their device memory from one stream-ordered pool
// per device that the library owns.  Freed blocks stay reserved in the pool
// up to its release threshold (16 GiB unless wbpr_memory_cache sets another),
// so a create / destroy cycle of the same size maps no new memory and frees
// nothing back to the driver: cudaFree of a few GB costs milliseconds, a
// pool free microseconds.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace wbpr {

// The pool of `device`, created on first use; nullptr if it cannot be made.
cudaMemPool_t device_pool(int device);

// `bytes` from the pool of the current device, ordered on `stream`, and
// usable from any stream on return (the allocation's own dependencies have
// completed).
cudaError_t pool_alloc(void** p, size_t bytes, cudaStream_t stream);

// `bytes` from the pool of the current device for use on `stream` only.
cudaError_t pool_alloc_on(void** p, size_t bytes, cudaStream_t stream);

}  // namespace wbpr
