// synth.cu -- deterministic synthetic int8 I/Q stream on the GPU.  Integer
// arithmetic only, so every sample equals the CPU generator's bit for bit:
//   sample(e, t) = clip(round((z_e(t) sigma_e + sum_k z_k(t - d_ke) sigma_k) M / 2^24
//                             + tone_e(t mod Nch)), -127, 127)          (Q16)
// z = sum of four 16-bit fields of a SplitMix64 hash of (time, stream,
// component) minus 131070 (Irwin-Hall, ~N(0, 37837^2)); M = 113512.
// Time t = s*Nch + c, the reference depacketiser's sample index
// (MDT_OneStation_client.cu:852-858).
#include "mdt_common.cuh"

namespace mdt {

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ long long gauss_int(uint64_t seed, long long t, int stream, int comp)
{
    uint64_t key = ((uint64_t)t << 14) | ((uint64_t)stream << 1) | (uint64_t)comp;
    uint64_t h = mix64(mix64(key) ^ seed);
    long long z = (long long)(h & 0xFFFF) + (long long)((h >> 16) & 0xFFFF) +
                  (long long)((h >> 32) & 0xFFFF) + (long long)(h >> 48);
    return z - 131070;
}

__global__ void synth_iq_kernel(uint64_t seed, int ne, int nch, long s0, long nsp,
                                const int32_t *__restrict__ sigma_q8,
                                const int32_t *__restrict__ tone_q16, int nsrc,
                                const int32_t *__restrict__ src_sigma_q8,
                                const int32_t *__restrict__ src_delay, char2 *out)
{
    const long total = nsp * ne * (long)nch;
    for (long idx = threadIdx.x + (long)blockIdx.x * blockDim.x; idx < total;
         idx += (long)gridDim.x * blockDim.x) {
        const long row = idx / nch;
        const int c = (int)(idx - row * nch);
        const long s = s0 + row / ne;
        const int e = (int)(row % ne);
        const long long t = (long long)s * nch + c;
        signed char v[2];
#pragma unroll
        for (int comp = 0; comp < 2; comp++) {
            long long num = gauss_int(seed, t, e, comp) * sigma_q8[e];
            for (int k = 0; k < nsrc; k++)
                num += gauss_int(seed, t - src_delay[k * ne + e], 4096 + k, comp) * src_sigma_q8[k];
            long long x = (num * 113512LL) >> 24;
            if (tone_q16) x += tone_q16[2 * ((long)e * nch + c) + comp];
            x = (x + 32768) >> 16;
            x = x > 127 ? 127 : (x < -127 ? -127 : x);
            v[comp] = (signed char)x;
        }
        out[idx] = make_char2(v[0], v[1]);
    }
}

}  // namespace mdt

extern "C" MDT_API mdt_status mdt_synth_iq(uint64_t seed, int ne, int nch, long s0, long nsp,
                                           const int32_t *sigma_q8, const int32_t *tone_q16,
                                           int nsrc, const int32_t *src_sigma_q8,
                                           const int32_t *src_delay, int8_t *out,
                                           cudaStream_t stream)
{
    if (ne <= 0 || ne >= 4096 || nch <= 0 || nsp < 0 || !sigma_q8 || !out || nsrc < 0 ||
        (nsrc > 0 && (!src_sigma_q8 || !src_delay)))
        return mdt::invalid("synth_iq: bad arguments");
    if (nsp == 0) return MDT_SUCCESS;
    long total = nsp * ne * (long)nch;
    long blocks = mdt::cdiv(total, 256);
    long cap = (long)mdt::sm_count() * 32;
    if (blocks > cap) blocks = cap;
    mdt::synth_iq_kernel<<<(unsigned)blocks, 256, 0, stream>>>(
        seed, ne, nch, s0, nsp, sigma_q8, tone_q16, nsrc, src_sigma_q8, src_delay,
        reinterpret_cast<char2 *>(out));
    return mdt::launch_status("synth_iq_kernel");
}
