// sr_wave_trace.cu — the wavefront traversal kernel (k_wave_trace, sr_wave_kernels.cuh) at block sizes
// other than the default 128 threads: 64 and 256, a run-time choice of the scene's tuning
// (SrTuning::trace_block_threads) that the autotuner sweeps.  Kept apart from sr_wavefront.cu so
// that the extra instantiations build in parallel with it.  Results do not depend on the block size
// (every query runs the same actions); work-counting renders use the default size.
#include <cuda_runtime.h>

#include "sr_wave_kernels.cuh"

namespace sr {

template <int BLOCK>
static void trace_at(const WaveLaunch& L, const WaveState& W, int cur, cudaStream_t st, bool loop_shadows) {
    if (L.general) {
        if (loop_shadows)
            k_wave_trace<false, true, false, BLOCK><<<L.grid_trace, BLOCK, 0, st>>>(W, L.S, cur, L.err, nullptr);
        else
            k_wave_trace<false, true, true, BLOCK><<<L.grid_trace, BLOCK, 0, st>>>(W, L.S, cur, L.err, nullptr);
    } else {
        k_wave_trace<false, false, true, BLOCK><<<L.grid_trace, BLOCK, 0, st>>>(W, L.S, cur, L.err, nullptr);
    }
}

void wave_trace_block(const WaveLaunch& L, const WaveState& W, int cur, cudaStream_t st, bool loop_shadows) {
    if (L.trace_block == 64)
        trace_at<64>(L, W, cur, st, loop_shadows);
    else
        trace_at<256>(L, W, cur, st, loop_shadows);
}

int wave_trace_occupancy(bool general, int block) {
    int b = 0;
    if (block == 64)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &b, general ? k_wave_trace<false, true, true, 64> : k_wave_trace<false, false, true, 64>, 64, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &b, general ? k_wave_trace<false, true, true, 256> : k_wave_trace<false, false, true, 256>, 256, 0);
    return b;
}

}  // namespace sr
