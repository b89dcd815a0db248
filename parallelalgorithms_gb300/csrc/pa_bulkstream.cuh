// Streaming a contiguous byte range through shared memory with bulk copies
// (the TMA engine's non-tensor form), for the read-once sum kernel.
//
// A CTA of CONSUMERS + 32 threads owns the chunks blockIdx.x, blockIdx.x +
// gridDim.x, ... of the range (CHUNK bytes each, the last one possibly
// shorter).  Lane 0 of the last warp is the producer: it issues one bulk
// copy per chunk into the next stage of a ring of STAGES shared-memory
// stages, completing on that stage's "full" mbarrier, after the consumers
// have released the stage's previous chunk on its "empty" mbarrier.  The
// CONSUMERS threads wait for each chunk, hand it to `consume`, and release
// the stage.  STAGES x CHUNK bytes are in flight per CTA, independent of
// registers, which is what a streaming read needs to reach HBM bandwidth.
//
// Every wait is bounded: a wait that gives up raises DEVERR_TMA_TIMEOUT in
// *err and stops the streaming (the CTA's result is then invalid, and the
// call reports the error).  A consumer warp leaves as a whole (so that no lane
// is left alone in a warp-collective `consume`), the producer stops issuing
// copies, and before the CTA exits the producer waits (bounded again) for the
// copies it issued into stages that no consumer has waited out, so that no
// copy lands in shared memory after the CTA is gone.
#pragma once

#include "pa_common.cuh"

namespace pa {

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

template <int STAGES, int CHUNK, int CONSUMERS>
struct BulkRing {
  static_assert(CHUNK % 16 == 0, "chunks are whole 16-byte vectors");
  static_assert(CONSUMERS % 32 == 0, "consumers are whole warps");
  static constexpr int kThreads = CONSUMERS + 32;
  static constexpr size_t kBarOff = (size_t)STAGES * CHUNK;
  static constexpr size_t kBytes = kBarOff + 2 * (size_t)STAGES * 8;
};

// `src` 16-byte aligned, `bytes` a multiple of 16; `ring` is
// BulkRing::kBytes of shared memory (16-byte aligned).  consume(stage, nvec)
// is called by every consumer thread (threadIdx.x < CONSUMERS) for each of
// the CTA's chunks, in order, with the chunk's nvec 16-byte vectors; it may
// use warp-collective operations (all lanes of a consumer warp call it the
// same number of times).  Called by all threads of the CTA; ends with a
// barrier.
template <int STAGES, int CHUNK, int CONSUMERS, typename F>
__device__ __forceinline__ void bulk_stream(const void* src, size_t bytes, unsigned char* ring, uint32_t* err,
                                            F&& consume) {
  using R = BulkRing<STAGES, CHUNK, CONSUMERS>;
  uint64_t* full = reinterpret_cast<uint64_t*>(ring + R::kBarOff);
  uint64_t* empty = full + STAGES;
  constexpr uint32_t kConsumerWarps = CONSUMERS / 32;
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kConsumerWarps);
    }
    mbar_fence_init();
  }
  __syncthreads();
  const size_t nchunks = (bytes + CHUNK - 1) / CHUNK;
  const size_t g = gridDim.x;
  const size_t mine = blockIdx.x < nchunks ? (nchunks - blockIdx.x + g - 1) / g : 0;
  const unsigned char* s8 = static_cast<const unsigned char*>(src);
  if (warp == kConsumerWarps) {
    if (lane == 0) {  // producer
      size_t issued = 0;
      for (size_t j = 0; j < mine; ++j) {
        const uint32_t s = (uint32_t)(j % STAGES);
        if (j >= (size_t)STAGES && !mbar_wait_bounded(&empty[s], (uint32_t)((j / STAGES) - 1) & 1u, err)) break;
        const size_t off = (blockIdx.x + j * g) * (size_t)CHUNK;
        const uint32_t len = (uint32_t)min((size_t)CHUNK, bytes - off);
        mbar_arrive_expect_tx(&full[s], len);
        bulk_load_g2s(ring + (size_t)s * CHUNK, s8 + off, len, &full[s]);
        issued = j + 1;
      }
      // Only the last STAGES issued copies can still be in flight (an earlier
      // stage was reused after its chunk was consumed); wait for their
      // phases, which returns at once for every copy that has landed.
      for (size_t j = issued > (size_t)STAGES ? issued - STAGES : 0; j < issued; ++j)
        if (!mbar_wait_bounded(&full[j % STAGES], (uint32_t)(j / STAGES) & 1u, err)) break;
    }
  } else {  // consumers
    for (size_t j = 0; j < mine; ++j) {
      const uint32_t s = (uint32_t)(j % STAGES);
      const size_t off = (blockIdx.x + j * g) * (size_t)CHUNK;
      const uint32_t len = (uint32_t)min((size_t)CHUNK, bytes - off);
      const bool landed = mbar_wait_bounded(&full[s], (uint32_t)(j / STAGES) & 1u, err);
      if (!__all_sync(0xFFFFFFFFu, landed)) break;  // the whole warp leaves together
      consume(reinterpret_cast<const uint4*>(ring + (size_t)s * CHUNK), len / 16u);
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
    }
  }
  __syncthreads();
}

}  // namespace pa
