// xengine_tc.cuh -- host-visible pieces of the tensor-core X-engine shared
// with the batch driver (batch.cu): tile and work descriptors.
#pragma once
#include "mdt_common.cuh"

namespace mdt {

struct TcTile {
    int16_t r0, q0, n, a_sep;  // row-tile start, column-chunk start, chunk width, A loaded apart
};

// One job of a batched X-engine launch.
struct XJob {
    const uint8_t *X;  // X16 operand of the job
    long chunk_bytes;  // stride between 32-spectrum chunks: Nch * NEp * 128
    long chan_bytes;   // stride between channels: NEp * 128
    int ne, nep, nkc;
    float alpha;       // 1 / (Nsp * scale^2)
    float2 *V;         // visibilities [nch][ne*ne]
};

// One work entry of a batched X-engine launch: a tile of one channel of one job.
struct XWork {
    int job, ch;
    TcTile tile;
};

constexpr int TCB_MAXW = 128;  // widest column chunk of the batched X-engine

// Lower-triangle tiles (row tiles of 128, column chunks of <= maxw) for NE
// elements padded to nep rows; returns the count or -1 if more than 160.
int make_tiles(int ne, int nep, int maxw, TcTile *tiles);
int x16_padded_rows(int ne);
int x16_chunks(int nsp);
mdt_status xengine_tc_batched(const XJob *jobs, const XWork *work, int nwork, int *err,
                              cudaStream_t stream);

}  // namespace mdt
