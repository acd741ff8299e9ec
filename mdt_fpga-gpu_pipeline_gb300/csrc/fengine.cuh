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
    int wk0;           // first work item of the job in a tensor-core F-engine launch
};

// Work items of one job in a tensor-core F-engine launch (runs of 512 spectra).
inline long fjob_tc_items(int ne, int nsp) { return (long)ne * ((nsp + 511) / 512); }
// Whether the tensor-core F-engine handles this shape.
inline bool fengine_tc_shape(int nch, int ntaps) { return nch == 1024 && (ntaps == 4 || ntaps == 8); }

// Blocks of one job in a batched launch: 4 per (element, 32-spectrum chunk).
inline long fjob_blocks(int ne, int nkc) { return (long)ne * nkc * 4; }

mdt_status fengine_x16_batched(int nch, int ntaps, const FJob *jobs, int njobs, long nblocks,
                               cudaStream_t stream);
// Batched tensor-core F-engine (f16 output) over jobs of Nch 1024 and one
// Ntaps (4 or 8); `jobs` is a device array with wk0 prefix sums, `nwork` the
// total work items.
mdt_status fengine_tc_batched(int ntaps, const FJob *jobs, int njobs, long nwork, int *err,
                              cudaStream_t stream);
// The FP32 path's F-output XB: complex64 in blocks of 8 spectra (ceil(Nsp/8)
// blocks, spectra past Nsp zero); every (block, channel, element) is one
// 64-byte run of the block's 8 spectra.  Block-major, XB[s/8][c][e][s%8], so an
// F-engine unit's runs for all its channels lie within one block's Nch*NE*64
// bytes (MDT_XB_BLOCK_MAJOR 0: channel-major XB[c][s/8][e][s%8]).
#ifndef MDT_XB_BLOCK_MAJOR
#define MDT_XB_BLOCK_MAJOR 1
#endif
// complex64 elements between consecutive channels / consecutive 8-spectrum blocks
__host__ __device__ inline long xb_chan_stride(int ne, int nch, long nsb)
{
    return MDT_XB_BLOCK_MAJOR ? (long)ne * 8 : nsb * ne * 8;
}
__host__ __device__ inline long xb_block_stride(int ne, int nch, long nsb)
{
    return MDT_XB_BLOCK_MAJOR ? (long)nch * ne * 8 : (long)ne * 8;
}

mdt_status check_dims(int ne, int nch, int ntaps, int nsp);
const float2 *fft_twiddles(int n, mdt_status *st);

}  // namespace mdt
