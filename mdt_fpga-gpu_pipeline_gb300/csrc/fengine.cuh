// fengine.cuh -- host-visible pieces of the F-engines shared with the batch
// driver (batch.cu).
#pragma once
#include "mdt_common.cuh"

namespace mdt {

// One job of a batched f16 F-engine launch.
struct FJob {
    const char2 *iq;   // Nsp + Ntaps - 1 spectra
    const float *win;  // Ntaps * Nch
    uint8_t *X16;      // X16 operand of the job
    int ne, nsp, nep, nkc;
    float scale;
    int blk0;          // first block of the job (prefix sum over the launch)
};

// Blocks of one job in a batched launch: 4 per (element, 32-spectrum chunk).
inline long fjob_blocks(int ne, int nkc) { return (long)ne * nkc * 4; }

mdt_status fengine_x16_batched(int nch, int ntaps, const FJob *jobs, int njobs, long nblocks,
                               cudaStream_t stream);
mdt_status check_dims(int ne, int nch, int ntaps, int nsp);
const float2 *fft_twiddles(int n, mdt_status *st);

}  // namespace mdt
