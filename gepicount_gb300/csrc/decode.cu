// Genotype loader kernels: PLINK .bed (2-bit calls) or the reference reader's
// row-major bit planes -> class-sorted device bit-planes (layout in device.cuh).
//
// Semantics follow BinPlinkReader::readData (src/reader/BinPlinkReader.h:
// 160-211): code 00 -> column-5 allele row, 10 -> both rows, 11 -> column-6
// allele row, 01 -> missing; valid = not missing.  Samples are gathered through
// a permutation `perm` (output sample slot -> input sample index, -1 = pad), so
// class 0 (phenotype 1) comes first, then class 1 (phenotype 2), each padded to
// a multiple of 128 samples; samples of any other phenotype are dropped.
//
// Bit order inside a 32-sample word is nibble-transposed: sample slot k of the
// word sits at bit 8*(k%4) + k/4.  Popcount counting is blind to the order;
// the tensor-core counting form uses it to turn 4 consecutive samples into the
// 4 bytes of an 8-bit MMA operand register with one shift and one AND.
//
// HBM-bound: reads N * ceil(S/4) bytes, writes 3 * N * Wp * 4 bytes.
#include <cuda_runtime.h>

#include <cstdint>

#include "device.cuh"

namespace gepi {

// Shared memory of decode_bed_kernel: the staged rows (+ up to 15 bytes of
// alignment offset), then the 33 x 32 permutation entries of 32 output words.
__host__ __device__ inline size_t decode_rows_bytes(int spc, size_t bps) {
    return ((size_t)spc * bps + 16 + 15) & ~size_t(15);
}
constexpr size_t kDecodePermBytes = 33 * 32 * 4;

// One CTA decodes `spc` consecutive SNPs whose .bed rows are staged in shared
// memory.  The rows are contiguous in the file, so the staging is one copy of
// spc * bps bytes: 16-byte loads, four in flight per thread (byte loads kept a
// warp at 32 bytes in flight, about 250 GB/s over the GPU), into a shared
// buffer offset to match the source's alignment (the payload follows a 3-byte
// header), with byte loads for the unaligned head and tail.
// Then, 32 output words at a time, the CTA stages those words' sample
// permutation in shared memory (32 x 32 entries, row pitch 33 so that the
// lanes' reads fall in distinct banks), and each warp produces the 32 words of
// one SNP: lane L builds word w0 + L of the three planes from its 32 slots,
// slot k at bit 8 (k % 4) + k / 4, and the warp stores them coalesced.
__global__ void decode_bed_kernel(const uint8_t *__restrict__ bed, size_t bps, int n_snps,
                                  const int32_t *__restrict__ perm, int Wp, int spc,
                                  uint32_t *__restrict__ planes) {
    extern __shared__ __align__(16) uint8_t sbuf[];
    const int s0 = blockIdx.x * spc;
    const int ns = min(spc, n_snps - s0);
    const size_t tot = (size_t)ns * bps;
    const uint8_t *src = bed + (size_t)s0 * bps;
    const int pad = (int)((uintptr_t)src & 15);
    uint8_t *srow = sbuf + pad;  // congruent with src modulo 16
    const size_t head = min((size_t)((16 - pad) & 15), tot);
    const size_t nvec = (tot - head) / 16;
    const size_t bd = blockDim.x;
    for (size_t i = threadIdx.x; i < head; i += bd) srow[i] = __ldg(src + i);
    {
        const uint4 *vs = reinterpret_cast<const uint4 *>(src + head);
        uint4 *vd = reinterpret_cast<uint4 *>(srow + head);
        size_t i = threadIdx.x;
        for (; i + 3 * bd < nvec; i += 4 * bd) {
            const uint4 v0 = __ldg(vs + i), v1 = __ldg(vs + i + bd), v2 = __ldg(vs + i + 2 * bd),
                        v3 = __ldg(vs + i + 3 * bd);
            vd[i] = v0;
            vd[i + bd] = v1;
            vd[i + 2 * bd] = v2;
            vd[i + 3 * bd] = v3;
        }
        for (; i < nvec; i += bd) vd[i] = __ldg(vs + i);
    }
    for (size_t i = head + nvec * 16 + threadIdx.x; i < tot; i += bd) srow[i] = __ldg(src + i);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    int32_t *sperm = reinterpret_cast<int32_t *>(sbuf + decode_rows_bytes(spc, bps));
    const int nchunks = (Wp + 31) / 32;
    for (int ch = 0; ch < nchunks; ++ch) {
        const int w0 = ch * 32;
        __syncthreads();  // the rows are staged; the previous chunk's readers are done
        for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
            const int w = w0 + (i >> 5);
            sperm[(i >> 5) * 33 + (i & 31)] = w < Wp ? __ldg(perm + (size_t)w0 * 32 + i) : -1;
        }
        __syncthreads();
        const int32_t *myperm = sperm + lane * 33;
        const int w = w0 + lane;
        for (int si = warp; si < ns; si += nwarp) {
            const uint8_t *row = srow + (size_t)si * bps;
            uint32_t A = 0, a = 0, V = 0;
#pragma unroll 8
            for (int k = 0; k < 32; ++k) {
                const int sample = myperm[k];
                int code = 1;  // pad slot: missing
                if (sample >= 0) code = (row[sample >> 2] >> ((sample & 3) * 2)) & 3;
                const uint32_t bit = 1u << (8 * (k & 3) + (k >> 2));
                A |= (code & 1) == 0 ? bit : 0u;  // 00, 10
                a |= code >= 2 ? bit : 0u;        // 10, 11
                V |= code != 1 ? bit : 0u;        // not 01
            }
            if (w < Wp) {
                uint32_t *out = planes + (size_t)(s0 + si) * 3 * Wp + w;
                out[0] = A;
                out[(size_t)Wp] = a;
                out[2 * (size_t)Wp] = V;
            }
        }
    }
}

// Same, from the reference reader's host rows (uploaded): bits/valid are
// rows x nw uint64 with sample j at bit j%64 of word j/64; allele rows 2s and
// 2s+1 share the valid row.  Bits are masked with valid, as every count of the
// reference is (proc_gold_1.h:106-112).
__global__ void decode_rows_kernel(const uint64_t *__restrict__ bits,
                                   const uint64_t *__restrict__ valid, int nw, int n_snps,
                                   const int32_t *__restrict__ perm, int Wp,
                                   uint32_t *__restrict__ planes) {
    const int lane = threadIdx.x & 31;
    const int slot = 4 * (lane & 7) + (lane >> 3);  // slot whose bit is `lane`
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarp = (gridDim.x * blockDim.x) >> 5;
    const int nchunks = (Wp + 31) / 32;
    for (long long job = gwarp; job < (long long)nchunks * n_snps; job += nwarp) {
        const int s = (int)(job / nchunks), ch = (int)(job - (long long)s * nchunks);
        const int w0 = ch * 32;
        const uint64_t *bA = bits + (size_t)(2 * s) * nw, *ba = bA + nw;
        const uint64_t *vv = valid + (size_t)(2 * s) * nw;
        uint32_t myA = 0, mya = 0, myV = 0;
        for (int j = 0; j < 32; ++j) {
            const int w = w0 + j;
            if (w >= Wp) break;
            const int sample = __ldg(perm + (size_t)w * 32 + slot);
            bool A = false, a = false, V = false;
            if (sample >= 0) {
                const int k = sample >> 6;
                const uint64_t bit = 1ull << (sample & 63);
                V = (__ldg(vv + k) & bit) != 0;
                A = V && (__ldg(bA + k) & bit) != 0;
                a = V && (__ldg(ba + k) & bit) != 0;
            }
            const uint32_t bAw = __ballot_sync(0xffffffffu, A);
            const uint32_t baw = __ballot_sync(0xffffffffu, a);
            const uint32_t bVw = __ballot_sync(0xffffffffu, V);
            if (lane == j) {
                myA = bAw;
                mya = baw;
                myV = bVw;
            }
        }
        const int w = w0 + lane;
        if (w < Wp) {
            uint32_t *out = planes + (size_t)s * 3 * Wp + w;
            out[0] = myA;
            out[(size_t)Wp] = mya;
            out[2 * (size_t)Wp] = myV;
        }
    }
}

cudaError_t launch_decode_bed(const uint8_t *bed_payload, size_t bps, int n_snps,
                              const int32_t *perm, int Wp, uint32_t *planes,
                              cudaStream_t stream) {
    if (n_snps <= 0) return cudaSuccess;
    const size_t budget = 40 * 1024;
    int spc = (int)(budget / (bps ? bps : 1));
    if (spc < 1) spc = 1;
    if (spc > 32) spc = 32;
    size_t smem = decode_rows_bytes(spc, bps) + kDecodePermBytes;
    if (smem > 200 * 1024) return cudaErrorInvalidValue;  // > ~800k samples: not supported
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(decode_bed_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    int grid = (n_snps + spc - 1) / spc;
    decode_bed_kernel<<<grid, 256, smem, stream>>>(bed_payload, bps, n_snps, perm, Wp, spc,
                                                   planes);
    return cudaGetLastError();
}

cudaError_t launch_decode_rows(const uint64_t *bits, const uint64_t *valid, int nw, int n_snps,
                               const int32_t *perm, int Wp, uint32_t *planes,
                               cudaStream_t stream, int num_sms) {
    if (n_snps <= 0) return cudaSuccess;
    long long jobs = (long long)((Wp + 31) / 32) * n_snps;
    long long blocks = (jobs + 7) / 8;
    long long cap = (long long)num_sms * 8;
    int grid = (int)(blocks < cap ? blocks : cap);
    if (grid < 1) grid = 1;
    decode_rows_kernel<<<grid, 256, 0, stream>>>(bits, valid, nw, n_snps, perm, Wp, planes);
    return cudaGetLastError();
}

// Marginal association of every SNP with the class: the larger phi^2 of its
// two allele rows' carrier x class tables (D^2 / ((a + b)(m - a - b) y z),
// D = a z - b y; a, b carriers and y, z valid samples of class 0, 1).  One
// warp per SNP.  The scan uses it only to order its tiles.
__global__ void marginal_kernel(const uint32_t *__restrict__ planes, int n_snps, int Wp, int W0,
                                float *__restrict__ score) {
    const int lane = threadIdx.x & 31;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarp = (gridDim.x * blockDim.x) >> 5;
    for (int s = gwarp; s < n_snps; s += nwarp) {
        const uint32_t *r = planes + (size_t)s * 3 * Wp;
        int c[3][2] = {{0, 0}, {0, 0}, {0, 0}};
        for (int w = lane; w < Wp; w += 32) {
            const int cls = w < W0 ? 0 : 1;
#pragma unroll
            for (int p = 0; p < 3; ++p) c[p][cls] += __popc(__ldg(r + (size_t)p * Wp + w));
        }
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int k = 0; k < 2; ++k)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) c[p][k] += __shfl_xor_sync(0xffffffffu, c[p][k], o);
        if (lane == 0) {
            const double y = c[2][0], z = c[2][1], m = y + z;
            double best = 0.0;
            for (int p = 0; p < 2; ++p) {
                const double a = c[p][0], b = c[p][1], n = a + b;
                const double den = n * (m - n) * y * z;
                if (den > 0.0) {
                    const double d = a * z - b * y;
                    best = fmax(best, d * d / den);
                }
            }
            score[s] = (float)best;
        }
    }
}

cudaError_t launch_marginal(const uint32_t *planes, int n_snps, int Wp, int W0, float *score,
                            int num_sms, cudaStream_t stream) {
    if (n_snps <= 0) return cudaSuccess;
    marginal_kernel<<<num_sms * 4, 256, 0, stream>>>(planes, n_snps, Wp, W0, score);
    return cudaGetLastError();
}

}  // namespace gepi
