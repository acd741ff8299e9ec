/*
 * ref_runner.cpp -- CPU grid runner for the reference kernels compiled from
 * the reference sources by oracle/build_ref.sh (PFB_Window_min4term_BH,
 * PpS_Batch, ReorderFOutput from MDT_OneStation_client/MDT_device_functions.cu).
 * Each launch walks the grid block by block; a block is one OpenMP team of
 * blockDim.x*blockDim.y*blockDim.z threads so that __syncthreads() (an omp
 * barrier) has CUDA semantics.  Test infrastructure only.
 */
#include <omp.h>
#include <stdio.h>

#include "mdt_cuda_emu.h"
#include "cufft.h"

thread_local mdt_emu_uint3 threadIdx;
thread_local mdt_emu_uint3 blockIdx;
mdt_emu_uint3 blockDim;
mdt_emu_uint3 gridDim;

/* Reference kernel prototypes (MDT_device_functions.h:44-46). */
void PFB_Window_min4term_BH(int, int, float *);
void PpS_Batch(int, int, float *, cuComplex *, cufftComplex *);
void ReorderFOutput(int, int, cufftComplex *, cuComplex *);

template <class F>
static int run_grid(unsigned gx, unsigned gy, unsigned gz, unsigned bx, unsigned by, unsigned bz,
                    F body)
{
    gridDim = {gx, gy, gz};
    blockDim = {bx, by, bz};
    const int nthr = (int)(bx * by * bz);
    int bad = 0;
    omp_set_dynamic(0);
    for (unsigned z = 0; z < gz; z++)
        for (unsigned y = 0; y < gy; y++)
            for (unsigned x = 0; x < gx; x++) {
                #pragma omp parallel num_threads(nthr)
                {
                    if (omp_get_num_threads() != nthr) {
                        #pragma omp atomic write
                        bad = 1;
                    } else {
                        unsigned t = (unsigned)omp_get_thread_num();
                        threadIdx = {t % bx, (t / bx) % by, t / (bx * by)};
                        blockIdx = {x, y, z};
                        body();
                    }
                }
                if (bad) return -1;
            }
    return 0;
}

extern "C" int ref_PFB_Window_min4term_BH(unsigned gx, unsigned bx, int nch, int ntaps, float *w)
{
    return run_grid(gx, 1, 1, bx, 1, 1, [&] { PFB_Window_min4term_BH(nch, ntaps, w); });
}

extern "C" int ref_PpS_Batch(unsigned gx, unsigned gy, unsigned gz, unsigned bx, int nch,
                             int ntaps, float *w, void *in, void *out)
{
    return run_grid(gx, gy, gz, bx, 1, 1, [&] {
        PpS_Batch(nch, ntaps, w, (cuComplex *)in, (cufftComplex *)out);
    });
}

extern "C" int ref_ReorderFOutput(unsigned gx, unsigned gy, unsigned gz, unsigned bx,
                                  unsigned by, int ne, int nch, void *F, void *X)
{
    return run_grid(gx, gy, gz, bx, by, 1, [&] {
        ReorderFOutput(ne, nch, (cufftComplex *)F, (cuComplex *)X);
    });
}
