// kernels.cu — ahead-of-time kernels of the expression path (nvcc, sm_103a).
//
//   ral_count_valid      null_count recount (GDFColumn.cu:519-529 uses cudf's
//                        gdf_count_nonzero_mask)
//   ral_gather_*         materialize_column (ColumnManipulation.cu:26-150): data
//                        gather plus validity gather with ballot-built words
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "device_rt.cuh"
#include "kernels.h"
#include "engine.h"

namespace ral {

namespace {

__global__ void count_valid_kernel(const ral_u32* __restrict__ valid, ral_i64 n, unsigned long long* out) {
    const ral_i64 words = (n + 31) >> 5;
    ral_u64 acc = 0;
    for (ral_i64 w = (ral_i64)blockIdx.x * blockDim.x + threadIdx.x; w < words; w += (ral_i64)gridDim.x * blockDim.x) {
        ral_u32 v = __ldg(valid + w);
        const ral_i64 rem = n - (w << 5);
        if (rem < 32) v &= (1u << rem) - 1u;
        acc += __popc(v);
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    __shared__ ral_u64 red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        ral_u64 t = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += red[k];
        if (t) atomicAdd(out, (unsigned long long)t);
    }
}

// One thread per output row; a warp builds each 32-row output validity word
// with a ballot, so there is no read-modify-write of shared words.
template <typename E, typename I>
__global__ void gather_kernel(const E* __restrict__ in, const ral_u32* __restrict__ in_valid, ral_i64 n_in,
                              const I* __restrict__ idx, ral_i64 n_out, E* __restrict__ out,
                              ral_u32* __restrict__ out_valid, unsigned long long* valid_count) {
    ral_u64 cnt = 0;
    const ral_i64 stride = (ral_i64)gridDim.x * blockDim.x;
    const ral_i64 n_round = (n_out + 31) & ~(ral_i64)31;
    for (ral_i64 i = (ral_i64)blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += stride) {
        bool bit = false;
        if (i < n_out) {
            const ral_i64 j = (ral_i64)idx[i];
            if (j >= 0 && j < n_in) {
                out[i] = in[j];
                bit = in_valid ? ((__ldg(in_valid + (j >> 5)) >> (j & 31)) & 1u) : true;
            }
        }
        if (out_valid) {
            const ral_u32 word = __ballot_sync(0xffffffffu, bit);
            if ((threadIdx.x & 31) == 0) {
                out_valid[i >> 5] = word;
                cnt += __popc(word);
            }
        }
    }
    if (valid_count) {
        for (int off = 16; off > 0; off >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, off);
        if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(valid_count, (unsigned long long)cnt);
    }
}

template <typename E>
cudaError_t gather_by_index(const void* in, const uint32_t* in_valid, int64_t n_in, const void* idx, int idx_width,
                            int64_t n_out,
                            void* out, uint32_t* out_valid, unsigned long long* valid_count, cudaStream_t st) {
    const int threads = 256;
    int64_t blocks = (n_out + threads - 1) / threads;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    const E* i_ = (const E*)in;
    E* o_ = (E*)out;
    switch (idx_width) {
    case 1: gather_kernel<E, int8_t><<<(int)blocks, threads, 0, st>>>(i_, in_valid, n_in, (const int8_t*)idx, n_out, o_, out_valid, valid_count); break;
    case 2: gather_kernel<E, int16_t><<<(int)blocks, threads, 0, st>>>(i_, in_valid, n_in, (const int16_t*)idx, n_out, o_, out_valid, valid_count); break;
    case 4: gather_kernel<E, int32_t><<<(int)blocks, threads, 0, st>>>(i_, in_valid, n_in, (const int32_t*)idx, n_out, o_, out_valid, valid_count); break;
    case 8: gather_kernel<E, int64_t><<<(int)blocks, threads, 0, st>>>(i_, in_valid, n_in, (const int64_t*)idx, n_out, o_, out_valid, valid_count); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}


// ---- every column of a frame gathered by one index column -----------------------------------
// A warp takes 128 consecutive output rows per step; lane t handles rows base + t + 32 k (k < 4),
// so each k is one coalesced index load, one coalesced store per column and one ballot-built
// validity word per nullable column, and every lane has eight independent loads in flight per
// column (four elements, four mask words).
//
// Two orders, chosen per launch from a sample of the index (every block computes the same choice):
// * clustered indices (a filter's kept rows, a sorted join side): row-major -- a step gathers every
//   column, so the index is read once and each column's nearby rows share cache lines;
// * scattered indices (an order-by permutation, a hash join): column-major -- the whole grid
//   gathers one column before the next.  Each column's random reads then stay within its own
//   span, and its validity mask (n/8 bytes) stays in L2 instead of competing with every other
//   column's mask; measured on six columns of 200M rows by a permutation, row-major took 48.7 ms
//   against 33.4 ms for six one-column passes.  The index is re-read per column (4 B per row).
// In the column-major order element loads are marked evict-first (`ld.global.cs`): a scattered
// element is read once, and the masks are what L2 should keep (clustered rows share lines, so the
// row-major order loads them normally).
constexpr int kGatherRowsPerLane = 4;
constexpr int kGatherSamples = 64;          // index samples of 32 consecutive rows
constexpr long long kGatherClusterSpan = 1 << 16;  // a sample spanning fewer input rows is clustered

template <typename I>
__device__ __forceinline__ ral_i64 ral_load_index(const void* idx, ral_i64 i) {
    return (ral_i64)__ldcs(reinterpret_cast<const I*>(idx) + i);
}

__device__ __forceinline__ ral_i64 ral_index_at(const GatherColumnsParams& P, ral_i64 i) {
    switch (P.idx_width) {
    case 1: return ral_load_index<int8_t>(P.idx, i);
    case 2: return ral_load_index<int16_t>(P.idx, i);
    case 4: return ral_load_index<int32_t>(P.idx, i);
    default: return ral_load_index<long long>(P.idx, i);
    }
}

// One column's step: the four element loads and the four validity-word loads are all issued before
// any is used (their values feed only the stores and ballots after them).
template <typename E, bool kScattered>
__device__ __forceinline__ unsigned ral_gather_k(const GatherColumn& c, const ral_i64 (&j)[kGatherRowsPerLane],
                                                 const bool (&ok)[kGatherRowsPerLane], ral_i64 base, int lane,
                                                 ral_i64 n_out) {
    const E* __restrict__ in = reinterpret_cast<const E*>(c.in);
    E* __restrict__ out = reinterpret_cast<E*>(c.out);
    const ral_u32* __restrict__ iv = c.in_valid;
    E v[kGatherRowsPerLane];
    ral_u32 w[kGatherRowsPerLane];
#pragma unroll
    for (int k = 0; k < kGatherRowsPerLane; ++k) {
        v[k] = ok[k] ? (kScattered ? __ldcs(in + j[k]) : __ldg(in + j[k])) : E(0);
        w[k] = ok[k] ? (iv ? __ldg(iv + (j[k] >> 5)) : 0xffffffffu) : 0u;
    }
#pragma unroll
    for (int k = 0; k < kGatherRowsPerLane; ++k)
        if (ok[k]) __stcs(out + base + lane + 32 * k, v[k]);
    unsigned cnt = 0;
    if (c.out_valid) {
#pragma unroll
        for (int k = 0; k < kGatherRowsPerLane; ++k) {
            const bool bit = (w[k] >> (j[k] & 31)) & 1u;
            const ral_u32 word = __ballot_sync(0xffffffffu, bit);
            // word k covers rows base + 32 k .. +31; lane k writes it (masks are padded to 64
            // bytes, so a partial last word stays inside the allocation)
            if (lane == k && base + 32 * k < n_out) c.out_valid[(base >> 5) + k] = word;
            cnt += __popc(word);
        }
    }
    return cnt;
}

template <bool kScattered>
__device__ __forceinline__ unsigned ral_gather_column_step(const GatherColumn& col, const ral_i64 (&j)[kGatherRowsPerLane],
                                                           const bool (&ok)[kGatherRowsPerLane], ral_i64 base,
                                                           int lane, ral_i64 n_out) {
    switch (col.width) {
    case 1: return ral_gather_k<int8_t, kScattered>(col, j, ok, base, lane, n_out);
    case 2: return ral_gather_k<short, kScattered>(col, j, ok, base, lane, n_out);
    case 4: return ral_gather_k<int, kScattered>(col, j, ok, base, lane, n_out);
    default: return ral_gather_k<long long, kScattered>(col, j, ok, base, lane, n_out);
    }
}

__device__ __forceinline__ void ral_step_indices(const GatherColumnsParams& P, ral_i64 base, int lane,
                                                 ral_i64 (&j)[kGatherRowsPerLane], bool (&ok)[kGatherRowsPerLane]) {
#pragma unroll
    for (int k = 0; k < kGatherRowsPerLane; ++k) {
        const ral_i64 i = base + lane + 32 * k;
        j[k] = i < P.n_out ? ral_index_at(P, i) : -1;
        ok[k] = j[k] >= 0 && j[k] < P.n_in;
    }
}

// Clustered samples among the 32 that warp `warp` (0 or 1) tests; kept out of line so that its
// registers do not add to the gather loops'.
__device__ __noinline__ int ral_gather_votes(const GatherColumnsParams& P, int warp, int lane) {
    int votes = 0;
    for (int q = warp * 32; q < warp * 32 + 32; ++q) {
        const ral_i64 at = (P.n_out - 32) / (kGatherSamples - 1) * q;
        const ral_i64 j = ral_index_at(P, at + lane);
        const bool in = j >= 0 && j < P.n_in;
        long long lo = in ? j : LLONG_MAX, hi = in ? j : LLONG_MIN;
        for (int off = 16; off > 0; off >>= 1) {
            lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, off));
            hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, off));
        }
        votes += (hi < lo || hi - lo < kGatherClusterSpan) ? 1 : 0;
    }
    return votes;
}

// 48 registers, five resident blocks of 256 threads per SM (a bound of six spills registers in the
// gather loops).
__global__ void __launch_bounds__(256, 5) gather_columns_kernel(const __grid_constant__ GatherColumnsParams P) {
    __shared__ unsigned long long s_cnt[kMaxGatherColumns];
    __shared__ int s_clustered;
    for (int c = threadIdx.x; c < P.num_columns; c += blockDim.x) s_cnt[c] = 0;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    // the order: warps 0 and 1 each test 32 samples of 32 consecutive indices (the same samples in
    // every block); a sample is clustered when its in-range indices span fewer than
    // kGatherClusterSpan input rows; a launch is clustered when at least half its samples are
    if (threadIdx.x == 0) s_clustered = 0;
    __syncthreads();
    if (P.num_columns > 1 && P.n_out >= 32 * kGatherSamples && warp < 2) {
        const int votes = ral_gather_votes(P, warp, lane);
        if (lane == 0) atomicAdd(&s_clustered, votes);
    }
    __syncthreads();
    const bool row_major = P.num_columns == 1 || P.n_out < 32 * kGatherSamples || 2 * s_clustered >= kGatherSamples;
    const ral_i64 step_rows = 32 * kGatherRowsPerLane;
    const ral_i64 nsteps = (P.n_out + step_rows - 1) / step_rows;
    const ral_i64 gwarp = ((ral_i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const ral_i64 nwarp = ((ral_i64)gridDim.x * blockDim.x) >> 5;
    if (row_major) {
        for (ral_i64 s = gwarp; s < nsteps; s += nwarp) {
            const ral_i64 base = s * step_rows;
            ral_i64 j[kGatherRowsPerLane];
            bool ok[kGatherRowsPerLane];
            ral_step_indices(P, base, lane, j, ok);
            for (int c = 0; c < P.num_columns; ++c) {
                const unsigned cnt = ral_gather_column_step<false>(P.col[c], j, ok, base, lane, P.n_out);
                if (lane == 0 && cnt) atomicAdd(&s_cnt[c], (unsigned long long)cnt);
            }
        }
    } else {
        for (int c = 0; c < P.num_columns; ++c) {
            unsigned long long cc = 0;
            for (ral_i64 s = gwarp; s < nsteps; s += nwarp) {
                const ral_i64 base = s * step_rows;
                ral_i64 j[kGatherRowsPerLane];
                bool ok[kGatherRowsPerLane];
                ral_step_indices(P, base, lane, j, ok);
                cc += ral_gather_column_step<true>(P.col[c], j, ok, base, lane, P.n_out);
            }
            if (lane == 0 && cc) atomicAdd(&s_cnt[c], cc);
        }
    }
    __syncthreads();
    if (P.valid_counts)
        for (int c = threadIdx.x; c < P.num_columns; c += blockDim.x)
            if (s_cnt[c]) atomicAdd(P.valid_counts + c, s_cnt[c]);
}

// ---- single-pass stream compaction (decoupled look-back) ---------------------------------
// Tile = 256 threads x 16 rows; the look-back is ral_lookback (device_rt.cuh).

__global__ void __launch_bounds__(256) compact_stencil_kernel(const int8_t* __restrict__ stencil,
                                                              const ral_u32* __restrict__ valid, ral_i64 n,
                                                              int32_t* __restrict__ out, ral_u64* scratch) {
    __shared__ ral_u32 s_tile;
    __shared__ ral_u32 s_warp[8];
    __shared__ ral_u64 s_prefix;
    ral_u64* status = scratch + 3;
    const ral_i64 ntiles = (n + kCompactTileRows - 1) / kCompactTileRows;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool vec_ok = (((uintptr_t)stencil) & 15) == 0;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd((unsigned int*)scratch, 1u);
        __syncthreads();
        const ral_i64 tile = s_tile;
        if (tile >= ntiles) break;
        const ral_i64 r0 = tile * kCompactTileRows + (ral_i64)threadIdx.x * 16;
        ral_u32 keep = 0;
        if (r0 + 16 <= n && vec_ok) {
            const uint4 v = __ldcs(reinterpret_cast<const uint4*>(stencil + r0));
            const ral_u32 w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int k = 0; k < 16; k++) keep |= (((w[k >> 2] >> (8 * (k & 3))) & 0xffu) != 0u ? 1u : 0u) << k;
        } else {
            for (int k = 0; k < 16; k++)
                if (r0 + k < n && stencil[r0 + k] != 0) keep |= 1u << k;
        }
        if (valid && r0 < n) keep &= (__ldg(valid + (r0 >> 5)) >> (r0 & 31)) & 0xffffu;
        const ral_u32 cnt = __popc(keep);
        ral_u32 incl = cnt;
        for (int off = 1; off < 32; off <<= 1) {
            const ral_u32 t = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += t;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            ral_u32 wv = lane < 8 ? s_warp[lane] : 0;
            ral_u32 wi = wv;
            for (int off = 1; off < 8; off <<= 1) {
                const ral_u32 t = __shfl_up_sync(0xffffffffu, wi, off);
                if (lane >= off) wi += t;
            }
            const ral_u32 total = __shfl_sync(0xffffffffu, wi, 7);
            const ral_u64 excl = ral_lookback(status, tile, total, scratch + 1);
            if (lane < 8) s_warp[lane] = wi - wv;
            if (lane == 0) {
                s_prefix = excl;
                if (tile == ntiles - 1) scratch[2] = excl + total;
            }
        }
        __syncthreads();
        ral_u64 pos = s_prefix + s_warp[warp] + (incl - cnt);
        while (keep) {
            const int k = __ffs(keep) - 1;
            keep &= keep - 1;
            out[pos++] = (int32_t)(r0 + k);
        }
        __syncthreads();
    }
}

}  // namespace

cudaError_t launch_count_valid(const uint32_t* valid, int64_t n, unsigned long long* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    int64_t words = (n + 31) / 32;
    int64_t blocks = (words + threads - 1) / threads;
    if (blocks > 152 * 8) blocks = 152 * 8;
    count_valid_kernel<<<(int)blocks, threads, 0, st>>>(valid, n, out);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_compact_stencil(const int8_t* stencil, const uint32_t* stencil_valid, int64_t n, int32_t* out_idx,
                                   unsigned long long* scratch, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int dev = 0, sms = 1, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, compact_stencil_kernel, 256, 0);
    if (per_sm < 1) per_sm = 1;
    const int64_t tiles = (n + kCompactTileRows - 1) / kCompactTileRows;
    int64_t grid = std::min<int64_t>(tiles, (int64_t)sms * per_sm);
    compact_stencil_kernel<<<(int)grid, 256, 0, st>>>(stencil, stencil_valid, n, out_idx, (ral_u64*)scratch);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_gather(int width, const void* in, const uint32_t* in_valid, int64_t n_in, const void* idx,
                          int idx_width, int64_t n_out, void* out, uint32_t* out_valid, unsigned long long* valid_count,
                          cudaStream_t st) {
    if (n_out <= 0) return cudaSuccess;
    switch (width) {
    case 1: return gather_by_index<int8_t>(in, in_valid, n_in, idx, idx_width, n_out, out, out_valid, valid_count, st);
    case 2: return gather_by_index<int16_t>(in, in_valid, n_in, idx, idx_width, n_out, out, out_valid, valid_count, st);
    case 4: return gather_by_index<int32_t>(in, in_valid, n_in, idx, idx_width, n_out, out, out_valid, valid_count, st);
    case 8: return gather_by_index<int64_t>(in, in_valid, n_in, idx, idx_width, n_out, out, out_valid, valid_count, st);
    default: return cudaErrorInvalidValue;
    }
}

namespace {
__global__ void category_insert_kernel(int32_t* __restrict__ codes, ral_i64 n, int32_t pos) {
    const ral_i64 stride = (ral_i64)gridDim.x * blockDim.x;
    for (ral_i64 i = (ral_i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        if (codes[i] >= pos) codes[i] += 1;
}
__global__ void category_remap_kernel(int32_t* __restrict__ codes, ral_i64 n, const int32_t* __restrict__ table,
                                      int32_t table_n) {
    const ral_i64 stride = (ral_i64)gridDim.x * blockDim.x;
    for (ral_i64 i = (ral_i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int32_t c = codes[i];
        if (c >= 0 && c < table_n) codes[i] = __ldg(table + c);
    }
}
}  // namespace

// ---- line index of a delimited text buffer ---------------------------------------------------
// Tile t of 64 KiB in 16 steps of 4 KiB: in step k, thread j reads bytes [16 j, 16 j + 16) of the
// step (one 16-byte load where the buffer allows it; a warp's loads are one contiguous 512 bytes),
// so a step's terminators come out in order from a block-wide scan of the threads' counts, and the
// steps in turn.

__device__ __forceinline__ ral_u32 ral_text_term_bits(const char* data, int64_t n, int64_t at, char term) {
    ral_u32 bits = 0;
    if (at + 16 <= n && ((uintptr_t)(data + at) & 15) == 0) {
        const uint4 v = __ldcs(reinterpret_cast<const uint4*>(data + at));
        const ral_u32 w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int k = 0; k < 16; ++k)
            bits |= ((ral_u32)(((w[k >> 2] >> (8 * (k & 3))) & 0xffu) == (ral_u32)(unsigned char)term)) << k;
    } else {
        for (int k = 0; k < 16; ++k)
            if (at + k < n && data[at + k] == term) bits |= 1u << k;
    }
    return bits;
}

__global__ void __launch_bounds__(256) text_term_count_kernel(const char* __restrict__ data, int64_t n, char term,
                                                              ral_u32* __restrict__ counts) {
    const int64_t tile = blockIdx.x;
    ral_u32 c = 0;
#pragma unroll 4
    for (int k = 0; k < (int)(kTextTileBytes / kTextStepBytes); ++k)
        c += __popc(ral_text_term_bits(data, n, tile * kTextTileBytes + k * kTextStepBytes + 16 * (int64_t)threadIdx.x, term));
    __shared__ ral_u32 s_w[8];
    const ral_u32 wsum = __reduce_add_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = wsum;
    __syncthreads();
    if (threadIdx.x == 0) {
        ral_u32 t = 0;
        for (int w = 0; w < 8; ++w) t += s_w[w];
        counts[tile] = t;
    }
}

__global__ void __launch_bounds__(1024) exclusive_scan_u32_kernel(const ral_u32* __restrict__ counts, int64_t m,
                                                                  unsigned long long* __restrict__ offsets) {
    __shared__ unsigned long long s_w[32];
    __shared__ unsigned long long s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t base = 0; base < m; base += 1024) {
        const int64_t i = base + threadIdx.x;
        const unsigned long long v = i < m ? counts[i] : 0ull;
        unsigned long long inc = v;
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned long long t = __shfl_up_sync(0xffffffffu, inc, off);
            if (lane >= off) inc += t;
        }
        if (lane == 31) s_w[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            unsigned long long w = s_w[lane];
            for (int off = 1; off < 32; off <<= 1) {
                const unsigned long long t = __shfl_up_sync(0xffffffffu, w, off);
                if (lane >= off) w += t;
            }
            s_w[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        const unsigned long long carry = s_carry;
        const unsigned long long before = (warp ? s_w[warp - 1] : 0ull) + inc - v;
        if (i < m) offsets[i] = carry + before;
        __syncthreads();
        if (threadIdx.x == 0) s_carry = carry + s_w[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) offsets[m] = s_carry;
}

__global__ void __launch_bounds__(256) text_term_positions_kernel(const char* __restrict__ data, int64_t n, char term,
                                                                  const unsigned long long* __restrict__ offsets,
                                                                  long long* __restrict__ ends) {
    const int64_t tile = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ ral_u32 s_w[2][8];
    unsigned long long base = offsets[tile];
    for (int k = 0; k < (int)(kTextTileBytes / kTextStepBytes); ++k) {
        const int64_t at = tile * kTextTileBytes + k * kTextStepBytes + 16 * (int64_t)threadIdx.x;
        if (tile * kTextTileBytes + k * kTextStepBytes >= n) break;  // block-uniform
        ral_u32 bits = ral_text_term_bits(data, n, at, term);
        const ral_u32 c = __popc(bits);
        ral_u32 inc = c;
        for (int off = 1; off < 32; off <<= 1) {
            const ral_u32 t = __shfl_up_sync(0xffffffffu, inc, off);
            if (lane >= off) inc += t;
        }
        if (lane == 31) s_w[k & 1][warp] = inc;  // double-buffered: no barrier between a step's reads and the next step's writes
        __syncthreads();
        ral_u32 before = inc - c, step_total = 0;
        for (int w = 0; w < 8; ++w) {
            const ral_u32 x = s_w[k & 1][w];
            if (w < warp) before += x;
            step_total += x;
        }
        unsigned long long q = base + before;
        for (; bits; bits &= bits - 1u) ends[q++] = at + __ffs(bits) - 1;
        base += step_total;
    }
}

__global__ void __launch_bounds__(256) text_present_count_kernel(const char* __restrict__ data, int64_t n,
                                                                 const long long* __restrict__ ends, int64_t nterm,
                                                                 int64_t lines, int64_t skip,
                                                                 unsigned long long* count) {
    ral_u32 c = 0;
    for (int64_t i = skip + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < lines;
         i += (int64_t)gridDim.x * blockDim.x) {
        const long long s = i == 0 ? 0 : ends[i - 1] + 1;
        long long e = i < nterm ? ends[i] : n;
        if (e > s && data[e - 1] == '\r') --e;
        c += e > s ? 1u : 0u;
    }
    c = __reduce_add_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, (unsigned long long)c);
}

cudaError_t launch_text_present_count(const char* data, int64_t n, const long long* ends, int64_t nterm, int64_t lines,
                                      int64_t skip, unsigned long long* count, cudaStream_t st) {
    if (lines <= skip) return cudaSuccess;
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((lines - skip + 255) / 256, 152 * 8));
    text_present_count_kernel<<<(int)blocks, 256, 0, st>>>(data, n, ends, nterm, lines, skip, count);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_text_term_counts(const char* data, int64_t n, char term, uint32_t* counts, cudaStream_t st) {
    const int64_t tiles = text_tiles(n);
    if (tiles <= 0) return cudaSuccess;
    if (tiles > 0x7fffffffll) return cudaErrorInvalidValue;
    text_term_count_kernel<<<(unsigned)tiles, 256, 0, st>>>(data, n, term, counts);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_exclusive_scan_u32(const uint32_t* counts, int64_t tiles, unsigned long long* offsets,
                                      cudaStream_t st) {
    exclusive_scan_u32_kernel<<<1, 1024, 0, st>>>(counts, tiles, offsets);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_text_term_positions(const char* data, int64_t n, char term, const unsigned long long* offsets,
                                       long long* ends, cudaStream_t st) {
    const int64_t tiles = text_tiles(n);
    if (tiles <= 0) return cudaSuccess;
    if (tiles > 0x7fffffffll) return cudaErrorInvalidValue;
    text_term_positions_kernel<<<(unsigned)tiles, 256, 0, st>>>(data, n, term, offsets, ends);
    note_launch();
    return cudaGetLastError();
}

// ---- Parquet data pages ----------------------------------------------------------------------
// A required column's page is its values back to back; an optional column's page starts with the
// 4-byte length of its definition levels (bit width 1) in the RLE / bit-packed hybrid (a run
// header varint h: h odd -> h >> 1 groups of 8 bit-packed levels, h even -> h >> 1 repeats of the
// next byte's level), then the values of the present rows only.  Two kernels:
//  * levels, one block per optional page: the level bytes are staged in shared memory, thread 0
//    turns the run headers into a table (a batch of up to kPqRuns runs at a time), and the block
//    writes the validity words from it, 32 rows per thread, counting the present rows of each
//    8192-row item; the counts become each item's first value index;
//  * values, one block per 8192-row item of a page: a required page copies its rows' values; an
//    optional page ranks each row among its item's present rows (a block scan of the validity
//    words' popcounts) and fetches its value.

constexpr int kPqRuns = 1024;
constexpr int kPqStage = 32768;  // level bytes of a page staged in shared memory

// An 8- or 4-byte little-endian value at base + i * w, where base has any alignment: two aligned
// loads and a funnel shift (the second load stays inside the 8-byte word holding the value's last
// byte, so it never leaves the buffer).
__device__ __forceinline__ unsigned long long ral_pq_value(const uint8_t* base, int64_t i, int w) {
    const uintptr_t a = (uintptr_t)(base + i * w);
    if (w == 8) {
        const int s = (int)(a & 7);
        const unsigned long long* q = reinterpret_cast<const unsigned long long*>(a - s);
        const unsigned long long lo = q[0];
        return s ? (lo >> (8 * s)) | (q[1] << (64 - 8 * s)) : lo;
    }
    const int s = (int)(a & 3);
    const ral_u32* q = reinterpret_cast<const ral_u32*>(a - s);
    const ral_u32 lo = q[0];
    return s ? (ral_u32)((lo >> (8 * s)) | (q[1] << (32 - 8 * s))) : lo;
}

__device__ __forceinline__ void ral_pq_store(void* base, int64_t i, int w, unsigned long long v) {
    if (w == 8) reinterpret_cast<unsigned long long*>(base)[i] = v;
    else reinterpret_cast<unsigned int*>(base)[i] = (unsigned int)v;
}

__global__ void __launch_bounds__(256) parquet_levels_kernel(const __grid_constant__ ParquetDecodeParams P) {
    __shared__ ral_u32 s_lw[kPqStage / 4 + 2];
    __shared__ int s_row[kPqRuns + 1];
    __shared__ int s_info[kPqRuns];  // bit-packed: byte offset of the run's levels; RLE: the level
    __shared__ unsigned char s_kind[kPqRuns];
    __shared__ int s_n, s_bad, s_emit, s_emit_end, s_done;
    __shared__ long long s_pos;
    const ParquetPage pg = P.pages[P.page_lo + blockIdx.x];
    if (!pg.optional || pg.rows <= 0) return;
    const ParquetColumnOut col = P.out[pg.column];
    const uint8_t* const lev = (const uint8_t*)pg.data + pg.lev_off;
    const int lev_bytes = pg.levels;
    const int off = (int)((uintptr_t)lev & 3);
    const int staged = min(lev_bytes, kPqStage);
    {
        // aligned words covering [lev, lev + staged): they stay inside the page's data or the
        // buffer's 16-byte padding
        const ral_u32* gw = reinterpret_cast<const ral_u32*>(lev - off);
        const int nw = (off + staged + 3) >> 2;
        for (int i = threadIdx.x; i < nw; i += blockDim.x) s_lw[i] = gw[i];
    }
    const uint8_t* const sb = reinterpret_cast<const uint8_t*>(s_lw) + off;
    auto lb = [&](long long p) -> unsigned long long {
        return p < staged ? sb[p] : (p < lev_bytes ? lev[p] : 0u);
    };
    if (threadIdx.x == 0) {
        s_pos = 0;
        s_n = 0;
        s_row[0] = 0;
        s_bad = 0;
        s_emit = 0;
        s_done = 0;
    }
    __syncthreads();
    const int words = (pg.rows + 31) >> 5;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    while (true) {
        if (threadIdx.x == 0) {
            // append runs after the carried ones; runs of no rows are skipped
            int k = s_n;
            int row = s_row[k];
            long long pos = s_pos;
            while (k < kPqRuns && row < pg.rows) {
                unsigned long long h = 0;
                int shift = 0;
                bool ok = true;
                while (true) {
                    if (pos >= lev_bytes || shift > 35) {
                        ok = false;
                        break;
                    }
                    const unsigned long long b = lb(pos++);
                    h |= (b & 0x7f) << shift;
                    shift += 7;
                    if (!(b & 0x80)) break;
                }
                if (!ok) {
                    s_bad = 1;
                    break;
                }
                int len;
                if (h & 1) {
                    const long long groups = (long long)(h >> 1);
                    if (pos + groups > lev_bytes) {
                        s_bad = 1;
                        break;
                    }
                    s_kind[k] = 1;
                    s_info[k] = (int)pos;
                    pos += groups;
                    len = (int)min((long long)pg.rows - row, groups * 8);
                } else {
                    if (pos >= lev_bytes) {
                        s_bad = 1;
                        break;
                    }
                    s_kind[k] = 0;
                    s_info[k] = (int)(lb(pos++) & 1);
                    len = (int)min((long long)pg.rows - row, (long long)(h >> 1));
                }
                if (len <= 0) continue;
                s_row[k] = row;
                row += len;
                ++k;
                s_row[k] = row;
            }
            s_pos = pos;
            s_n = k;
            // whole words covered by the table (all of them once the page's rows are)
            s_emit_end = row >= pg.rows ? words : (row >> 5);
        }
        __syncthreads();
        if (s_bad) break;
        const int n = s_n, e0 = s_emit, e1 = s_emit_end;
        for (int k0 = e0; k0 < e1; k0 += 256) {
            const int k = k0 + (int)threadIdx.x;
            ral_u32 X = 0;
            if (k < e1) {
                const int r0 = 32 * k, r1 = min(r0 + 32, pg.rows);
                int a = 0, b = n - 1;  // the last run starting at or before r0
                while (a < b) {
                    const int m = (a + b + 1) >> 1;
                    if (s_row[m] <= r0) a = m;
                    else b = m - 1;
                }
                for (int r = r0; r < r1; ++a) {
                    const int re = min(s_row[a + 1], r1);
                    const int len = re - r;
                    const ral_u32 m = len == 32 ? 0xffffffffu : ((1u << len) - 1u);
                    ral_u32 bits;
                    if (s_kind[a]) {
                        const int bo = r - s_row[a];
                        const long long p = s_info[a] + (bo >> 3);
                        const unsigned long long v = lb(p) | lb(p + 1) << 8 | lb(p + 2) << 16 | lb(p + 3) << 24 | lb(p + 4) << 32;
                        bits = (ral_u32)(v >> (bo & 7)) & m;
                    } else {
                        bits = s_info[a] ? m : 0u;
                    }
                    X |= bits << (r - r0);
                    r = re;
                }
            }
            // present rows per item (a warp's 32 words lie in at most two items)
            const int first = (k0 + 32 * warp) >> 8;
            const ral_u32 c = __popc(X);
            const ral_u32 ca = (k >> 8) == first ? c : 0u;
            const ral_u32 sa = __reduce_add_sync(0xffffffffu, ca);
            const ral_u32 sb2 = __reduce_add_sync(0xffffffffu, c - ca);
            if (lane == 0) {
                if (sa) atomicAdd(P.item_base + pg.item0 + first, sa);
                if (sb2) atomicAdd(P.item_base + pg.item0 + first + 1, sb2);
            }
            if (X) {
                const int64_t g = pg.row_start + 32 * (int64_t)k;
                const int sh = (int)(g & 31);
                ral_u32* const vw = col.valid + (g >> 5);
                if (sh == 0 && 32 * k + 32 <= pg.rows) {
                    *vw = X;  // the word holds rows of this page only
                } else {
                    atomicOr(vw, X << sh);
                    const ral_u32 hi = sh ? X >> (32 - sh) : 0u;
                    if (hi) atomicOr(vw + 1, hi);
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            s_emit = e1;
            if (e1 >= words) {
                s_done = 1;
            } else {
                // carry the runs that reach into the first word not written yet
                const int from = 32 * e1;
                int a = 0;
                while (a < n && s_row[a + 1] <= from) ++a;
                for (int j = a; j <= n; ++j) {
                    s_row[j - a] = s_row[j];
                    if (j < n) {
                        s_kind[j - a] = s_kind[j];
                        s_info[j - a] = s_info[j];
                    }
                }
                s_n = n - a;
            }
        }
        __syncthreads();
        if (s_done) break;
    }
    if (threadIdx.x == 0) {
        if (s_bad) {
            atomicAdd(P.status, 1ull);
            P.page_present[P.page_lo + blockIdx.x] = 0u;  // no indices are read for this page
            return;
        }
        // item counts -> each item's first value index; the page's values must cover them
        const int items = (pg.rows + kParquetItemRows - 1) / kParquetItemRows;
        ral_u32 run = 0;
        for (int i = 0; i < items; ++i) {
            const ral_u32 c = __ldcg(P.item_base + pg.item0 + i);
            P.item_base[pg.item0 + i] = run;
            run += c;
        }
        // PLAIN values must cover the present rows (a dictionary page's indices are checked by
        // their own kernel)
        const int64_t nvals = (pg.data_bytes - (int64_t)pg.values_off) / col.width;
        if (pg.dict_count == 0 && (int64_t)run > nvals) atomicAdd(P.status, 1ull);
        P.page_present[P.page_lo + blockIdx.x] = run;
        if (run) atomicAdd(P.status + 1 + pg.column, (unsigned long long)run);
    }
}

__global__ void __launch_bounds__(256) parquet_values_kernel(const __grid_constant__ ParquetDecodeParams P) {
    __shared__ ral_u32 s_word[256];
    __shared__ ral_u32 s_base[256];
    __shared__ ral_u32 s_wsum[8];
    const int item = P.item_lo + (int)blockIdx.x;
    int a = P.page_lo, b = P.page_hi - 1;  // the last page whose first item is at or before this one
    while (a < b) {
        const int m = (a + b + 1) >> 1;
        if (P.pages[m].item0 <= item) a = m;
        else b = m - 1;
    }
    const ParquetPage pg = P.pages[a];
    const ParquetColumnOut col = P.out[pg.column];
    const int w = col.width;
    const int rel0 = (item - pg.item0) * kParquetItemRows;
    const int rel1 = min(rel0 + kParquetItemRows, pg.rows);
    const int64_t lo = pg.values_off;
    const uint8_t* const vals = (const uint8_t*)pg.data + lo;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (pg.dict_count > 0 && !pg.optional) {
        // a dictionary-encoded required page: row r's entry is idx[idx0 + r] (checked in range)
        const uint8_t* const dict = (const uint8_t*)pg.dict;
        const uint32_t* const ix = P.idx + pg.idx0;
        for (int r = rel0 + (int)threadIdx.x; r < rel1; r += 256) {
            const uint32_t k = ix[r];  // in range unless the page was malformed (then reported)
            unsigned long long x = 0;
            if (k < (uint32_t)pg.dict_count) x = ral_pq_value(dict, k, w);
            ral_pq_store(col.data, pg.row_start + r, w, x);
        }
        return;
    }
    if (!pg.optional) {
        // Every row has its value (the page's length is checked on the host).  The lanes of a
        // warp take consecutive rows: each loads the aligned word where its value starts and
        // takes the next word from the lane after it (the last lane of the run loads it), so a
        // warp reads one contiguous aligned span whatever the values' alignment.
        const uintptr_t va = (uintptr_t)vals;
        if (w == 8) {
            // 16-byte words: lane l takes rows 2m, 2m + 1 (m = the warp's pair + l), bytes
            // [s + 16m, s + 16m + 16) past the aligned base: word m and, when s > 0, word m + 1
            // from the next lane (the last lane of the run loads it, when its values reach it)
            const int s16 = (int)(va & 15);
            const int k = s16 >> 2, f = (s16 & 3) * 8;
            const uint4* q = reinterpret_cast<const uint4*>(va - s16);
            unsigned long long* out = reinterpret_cast<unsigned long long*>(col.data) + pg.row_start;
#pragma unroll 2
            for (int m0 = (rel0 >> 1) + 32 * warp; 2 * m0 < rel1; m0 += 256) {
                const int m = m0 + lane;
                const int r = 2 * m;
                const bool in = r < rel1;
                const uint4 a = in ? q[m] : make_uint4(0u, 0u, 0u, 0u);
                uint4 b;
                b.x = __shfl_down_sync(0xffffffffu, a.x, 1);
                b.y = __shfl_down_sync(0xffffffffu, a.y, 1);
                b.z = __shfl_down_sync(0xffffffffu, a.z, 1);
                b.w = __shfl_down_sync(0xffffffffu, a.w, 1);
                const bool two = r + 1 < rel1;
                if (in && (lane == 31 || r + 2 >= rel1) && s16 + (two ? 16 : 8) > 16) b = q[m + 1];
                ral_u32 o0, o1, o2, o3;
                switch (k) {  // uniform over the page
                case 0: o0 = a.x; o1 = a.y; o2 = a.z; o3 = a.w; if (f) { o0 = __funnelshift_r(a.x, a.y, f); o1 = __funnelshift_r(a.y, a.z, f); o2 = __funnelshift_r(a.z, a.w, f); o3 = __funnelshift_r(a.w, b.x, f); } break;
                case 1: o0 = __funnelshift_r(a.y, a.z, f); o1 = __funnelshift_r(a.z, a.w, f); o2 = __funnelshift_r(a.w, b.x, f); o3 = __funnelshift_r(b.x, b.y, f); break;
                case 2: o0 = __funnelshift_r(a.z, a.w, f); o1 = __funnelshift_r(a.w, b.x, f); o2 = __funnelshift_r(b.x, b.y, f); o3 = __funnelshift_r(b.y, b.z, f); break;
                default: o0 = __funnelshift_r(a.w, b.x, f); o1 = __funnelshift_r(b.x, b.y, f); o2 = __funnelshift_r(b.y, b.z, f); o3 = __funnelshift_r(b.z, b.w, f); break;
                }
                if (in) out[r] = (unsigned long long)o1 << 32 | o0;
                if (two) out[r + 1] = (unsigned long long)o3 << 32 | o2;
            }
        } else {
            const int sh = (int)(va & 3) * 8;
            const ral_u32* q = reinterpret_cast<const ral_u32*>(va - (va & 3));
            ral_u32* out = reinterpret_cast<ral_u32*>(col.data) + pg.row_start;
#pragma unroll 4
            for (int r0 = rel0 + 32 * warp; r0 < rel1; r0 += 256) {
                const int r = r0 + lane;
                const bool in = r < rel1;
                const ral_u32 lo = in ? q[r] : 0u;
                ral_u32 nx = __shfl_down_sync(0xffffffffu, lo, 1);
                if (sh && in && (lane == 31 || r + 1 >= rel1)) nx = q[r + 1];
                if (in) out[r] = sh ? (lo >> sh) | (nx << (32 - sh)) : lo;
            }
        }
        return;
    }
    // PLAIN values, or a dictionary's entries through the present rows' indices
    const int64_t nvals = pg.dict_count > 0 ? (int64_t)0x7fffffffffffffffll : (pg.data_bytes - lo) / w;
    const uint8_t* const dict = (const uint8_t*)pg.dict;
    const uint32_t* const ix = P.idx + pg.idx0;
    // this item's validity words, page-relative (rows of the next page masked off)
    ral_u32 X = 0;
    {
        const int r0 = rel0 + 32 * (int)threadIdx.x;
        if (r0 < rel1) {
            const int64_t g = pg.row_start + r0;
            const int sh = (int)(g & 31);
            const int nb = min(32, rel1 - r0);
            const ral_u32* vw = col.valid + (g >> 5);
            X = vw[0] >> sh;
            if (sh && nb > 32 - sh) X |= vw[1] << (32 - sh);
            if (nb < 32) X &= (1u << nb) - 1u;
        }
    }
    // exclusive scan of the words' popcounts
    const ral_u32 c = __popc(X);
    ral_u32 incl = c;
    for (int d = 1; d < 32; d <<= 1) {
        const ral_u32 y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
    }
    if (lane == 31) s_wsum[warp] = incl;
    s_word[threadIdx.x] = X;
    __syncthreads();
    ral_u32 before = 0;
    for (int k = 0; k < warp; ++k) before += s_wsum[k];
    s_base[threadIdx.x] = before + incl - c;
    __syncthreads();
    const int64_t base = (int64_t)P.item_base[item];
    // each warp takes one word (32 rows) per step
    for (int t = warp; t * 32 < rel1 - rel0; t += 8) {
        const int r = rel0 + 32 * t + lane;
        if (r >= rel1) break;
        const ral_u32 Xw = s_word[t];
        unsigned long long x = 0;
        if ((Xw >> lane) & 1u) {
            const int64_t vi = base + s_base[t] + __popc(Xw & ((1u << lane) - 1u));
            if (pg.dict_count > 0) {
                const uint32_t k = ix[vi];
                if (k < (uint32_t)pg.dict_count) x = ral_pq_value(dict, k, w);
            }
            else if (vi < nvals) x = ral_pq_value(vals, vi, w);
        }
        ral_pq_store(col.data, pg.row_start + r, w, x);
    }
}

// One block per dictionary-encoded page: after the bit width byte, the present rows' indices in
// the RLE / bit-packed hybrid (a run header varint h: h odd -> (h >> 1) groups of 8 values of the
// bit width, packed from the low bits; h even -> h >> 1 repeats of the next ceil(width / 8) bytes).
// Thread 0 walks the run headers into a batch of segments (an RLE run, or up to kDictStage bytes of
// a bit-packed run: a long run is cut at group boundaries), the block copies the batch's span of
// packed bytes into shared memory with 16-byte loads, then writes the batch's indices from there,
// each checked against the dictionary's size.

constexpr int kDictStage = 32768;  // packed index bytes staged per batch
constexpr int kDictThreads = 1024;

__global__ void __launch_bounds__(kDictThreads) parquet_dict_index_kernel(const __grid_constant__ ParquetDecodeParams P) {
    __shared__ __align__(16) uint8_t s_buf[kDictStage + 64];
    __shared__ int s_row[kPqRuns + 1];
    __shared__ long long s_info[kPqRuns];  // bit-packed: stream offset of the segment's first value; RLE: the value
    __shared__ unsigned char s_kind[kPqRuns];
    __shared__ int s_n, s_bad, s_done;
    __shared__ long long s_pos, s_rem_groups, s_rem_pos, s_span0, s_span1;
    const int p = P.page_lo + (int)blockIdx.x;
    const ParquetPage pg = P.pages[p];
    if (pg.dict_count <= 0 || pg.rows <= 0) return;
    const int n_idx = pg.optional ? (int)min((unsigned)pg.rows, P.page_present[p]) : pg.rows;
    const uint8_t* const sv = (const uint8_t*)pg.data + pg.values_off;
    const long long sbytes = (long long)pg.data_bytes - pg.values_off;
    uint32_t* const ix = P.idx + pg.idx0;
    if (n_idx <= 0) return;
    if (sbytes < 1 || sv[0] > 32) {
        if (threadIdx.x == 0) atomicAdd(P.status, 1ull);
        return;
    }
    const int bw = sv[0];
    const int vbytes = (bw + 7) >> 3;
    const uint8_t* const st = sv + 1;
    const long long nb = sbytes - 1;
    const unsigned long long mask = bw == 32 ? 0xffffffffull : ((1ull << bw) - 1ull);
    // groups of one bit-packed segment: a batch's span stays within the stage
    const long long seg_groups = bw > 0 ? (long long)(kDictStage - 32) / bw : (1ll << 40);
    if (threadIdx.x == 0) {
        s_pos = 0;
        s_row[0] = 0;
        s_bad = 0;
        s_done = 0;
        s_rem_groups = 0;
        s_rem_pos = 0;
    }
    __syncthreads();
    while (true) {
        if (threadIdx.x == 0) {
            int k = 0;
            int row = s_row[0];
            long long pos = s_pos, rem = s_rem_groups, rpos = s_rem_pos;
            long long span0 = -1, span1 = -1;
            while (k < kPqRuns && row < n_idx) {
                if (rem > 0) {
                    // the next segment of the bit-packed run in progress
                    if (span0 < 0) span0 = rpos;
                    const long long room = (long long)(kDictStage - 32) - (rpos - span0);
                    long long g = bw > 0 ? min(rem, room / bw) : rem;
                    g = min(g, seg_groups);
                    if (g <= 0) break;  // the stage is full: the next batch goes on from here
                    const long long len = min(g * 8, (long long)(n_idx - row));
                    s_kind[k] = 1;
                    s_info[k] = rpos;
                    s_row[k] = row;
                    row += (int)len;
                    ++k;
                    s_row[k] = row;
                    rpos += g * bw;
                    span1 = rpos;
                    rem -= g;
                    continue;
                }
                unsigned long long h = 0;
                int shift = 0;
                bool ok = true;
                while (true) {
                    if (pos >= nb || shift > 35) {
                        ok = false;
                        break;
                    }
                    const unsigned long long b = st[pos++];
                    h |= (b & 0x7f) << shift;
                    shift += 7;
                    if (!(b & 0x80)) break;
                }
                if (!ok) {
                    s_bad = 1;
                    break;
                }
                if (h & 1) {
                    const long long groups = (long long)(h >> 1);
                    if (pos + groups * bw > nb) {
                        s_bad = 1;
                        break;
                    }
                    rem = groups;
                    rpos = pos;
                    pos += groups * bw;
                } else {
                    if (pos + vbytes > nb) {
                        s_bad = 1;
                        break;
                    }
                    unsigned long long v = 0;
                    for (int j = 0; j < vbytes; ++j) v |= (unsigned long long)st[pos + j] << (8 * j);
                    pos += vbytes;
                    const long long len = min((long long)(h >> 1), (long long)(n_idx - row));
                    if (len <= 0) continue;
                    s_kind[k] = 0;
                    s_info[k] = (long long)(v & mask);
                    s_row[k] = row;
                    row += (int)len;
                    ++k;
                    s_row[k] = row;
                }
            }
            s_pos = pos;
            s_rem_groups = row >= n_idx ? 0 : rem;
            s_rem_pos = rpos;
            s_n = k;
            s_span0 = span0;
            s_span1 = span1;
            if (row >= n_idx) s_done = 1;
            else if (k == 0 && !s_bad) s_bad = 1;
        }
        __syncthreads();
        if (s_bad) break;
        const int n = s_n, r_lo = s_row[0], r_hi = s_row[n];
        // the batch's packed bytes [span0, span1) into the stage: 16-byte loads from the aligned
        // address at or before them (inside the page's buffer, which is 16-byte padded)
        const long long span0 = s_span0, span1 = s_span1;
        long long sbase = 0;
        if (span0 >= 0) {
            const uintptr_t a0 = (uintptr_t)(st + span0) & ~(uintptr_t)15;
            const uintptr_t a1 = ((uintptr_t)(st + span1) + 15) & ~(uintptr_t)15;
            const int nv = (int)((a1 - a0) >> 4);
            for (int i = threadIdx.x; i < nv; i += blockDim.x)
                reinterpret_cast<uint4*>(s_buf)[i] = reinterpret_cast<const uint4*>(a0)[i];
            sbase = (long long)(a0 - (uintptr_t)st);  // stream offset of s_buf[0] (may be negative)
        }
        __syncthreads();
        for (int i = r_lo + (int)threadIdx.x; i < r_hi; i += kDictThreads) {
            int a = 0, b = n - 1;  // the last segment starting at or before i
            while (a < b) {
                const int m = (a + b + 1) >> 1;
                if (s_row[m] <= i) a = m;
                else b = m - 1;
            }
            unsigned long long v;
            if (s_kind[a]) {
                const long long bo = (long long)(i - s_row[a]) * bw;
                const long long q = s_info[a] + (bo >> 3) - sbase;  // in the stage
                unsigned long long x = 0;
#pragma unroll
                for (int j = 0; j < 5; ++j) x |= (unsigned long long)s_buf[q + j] << (8 * j);
                v = (x >> (bo & 7)) & mask;
            } else {
                v = (unsigned long long)s_info[a];
            }
            if (v >= (unsigned long long)pg.dict_count) {
                s_bad = 1;  // benign race: any writer sets it
                v = 0;
            }
            ix[i] = (uint32_t)v;
        }
        __syncthreads();
        if (s_bad || s_done) break;
        if (threadIdx.x == 0) s_row[0] = r_hi;
        __syncthreads();
    }
    if (threadIdx.x == 0 && s_bad) atomicAdd(P.status, 1ull);
}

cudaError_t launch_parquet_dict_indices(const ParquetDecodeParams& p, cudaStream_t st) {
    if (p.page_hi <= p.page_lo) return cudaSuccess;
    parquet_dict_index_kernel<<<p.page_hi - p.page_lo, kDictThreads, 0, st>>>(p);
    note_launch();
    return cudaGetLastError();
}

// ---- Snappy --------------------------------------------------------------------------------
// The raw Snappy format (google/snappy format_description.txt): a varint of the uncompressed
// length, then elements, each a tag byte whose low two bits give its kind: 0 a literal (length - 1
// in the tag's upper six bits, or for 60 .. 63 in the next 1 .. 4 bytes, little-endian), followed by
// its bytes; 1 a copy of 4 + ((tag >> 2) & 7) bytes from offset ((tag >> 5) << 8 | next byte);
// 2 and 3 a copy of 1 + (tag >> 2) bytes from a 2- or 4-byte little-endian offset.  A copy reads
// the output `offset` bytes back and may overlap itself (byte i reads byte i - offset).
// One warp per page: every lane decodes the same tags from a window of the input staged in shared
// memory (so control flow stays uniform), and the lanes move an element's bytes together: byte i of
// a copy is output[op - offset + i % offset], which precedes op, so one pass suffices.

constexpr int kSnapWin = 2048;

__global__ void __launch_bounds__(256) snappy_decompress_kernel(const SnappyJob* __restrict__ jobs, int32_t n_jobs,
                                                                unsigned long long* status) {
    __shared__ uint8_t s_win[8][kSnapWin];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j = (int)blockIdx.x * 8 + warp;
    if (j >= n_jobs) return;
    const SnappyJob job = jobs[j];
    uint8_t* const win = s_win[warp];
    for (int i = lane; i < job.prefix; i += 32) job.dst[i] = job.src[i - job.prefix];
    uint8_t* const out = job.dst + job.prefix;
    const uint8_t* const in = job.src;
    const int nin = job.src_bytes, nout = job.dst_bytes;
    int wbase = 0;
    auto load = [&](int at) {
        __syncwarp();
        for (int i = lane; i < kSnapWin; i += 32) win[i] = at + i < nin ? in[at + i] : 0;
        __syncwarp();
        wbase = at;
    };
    auto inb = [&](int q) -> unsigned {
        return (q >= wbase && q < wbase + kSnapWin) ? (unsigned)win[q - wbase] : (q < nin ? (unsigned)in[q] : 0u);
    };
    load(0);
    bool bad = false;
    int ip = 0, op = 0;
    {
        unsigned long long ulen = 0;
        int shift = 0;
        while (true) {
            if (ip >= nin || shift > 35) {
                bad = true;
                break;
            }
            const unsigned b = inb(ip++);
            ulen |= (unsigned long long)(b & 0x7f) << shift;
            shift += 7;
            if (!(b & 0x80)) break;
        }
        if (ulen != (unsigned long long)nout) bad = true;
    }
    while (!bad && ip < nin) {
        if (ip + 5 > wbase + kSnapWin) load(ip);  // the tag and its extra bytes in the window
        const unsigned tag = inb(ip);
        int len = 0, off = 0;
        const unsigned kind = tag & 3u;
        if (kind == 0u) {
            const unsigned l = tag >> 2;
            if (l < 60u) {
                len = (int)l + 1;
                ip += 1;
            } else {
                const int nb = (int)l - 59;
                unsigned long long v = 0;
                for (int k = 0; k < nb; ++k) v |= (unsigned long long)inb(ip + 1 + k) << (8 * k);
                if (ip + 1 + nb > nin || v >= 0x7fffffffull) {
                    bad = true;
                    break;
                }
                len = (int)v + 1;
                ip += 1 + nb;
            }
            if (len > nin - ip || len > nout - op) {
                bad = true;
                break;
            }
            for (int i = lane; i < len; i += 32) out[op + i] = (uint8_t)inb(ip + i);
            ip += len;
        } else {
            if (kind == 1u) {
                len = 4 + (int)((tag >> 2) & 7u);
                off = (int)(((tag >> 5) << 8) | inb(ip + 1));
                ip += 2;
            } else if (kind == 2u) {
                len = 1 + (int)(tag >> 2);
                off = (int)(inb(ip + 1) | inb(ip + 2) << 8);
                ip += 3;
            } else {
                len = 1 + (int)(tag >> 2);
                const unsigned long long o = (unsigned long long)inb(ip + 1) | (unsigned long long)inb(ip + 2) << 8 |
                                             (unsigned long long)inb(ip + 3) << 16 | (unsigned long long)inb(ip + 4) << 24;
                if (o > 0x7fffffffull) {
                    bad = true;
                    break;
                }
                off = (int)o;
                ip += 5;
            }
            if (ip > nin || off == 0 || off > op || len > nout - op) {
                bad = true;
                break;
            }
            __syncwarp();  // the bytes it reads, written by any lane, are visible
            for (int i = lane; i < len; i += 32) out[op + i] = out[op - off + i % off];
        }
        op += len;
        __syncwarp();
    }
    if (op != nout) bad = true;
    if (bad && lane == 0) atomicAdd(status, 1ull);
}

cudaError_t launch_snappy_decompress(const SnappyJob* jobs, int32_t n_jobs, unsigned long long* status, cudaStream_t st) {
    if (n_jobs <= 0) return cudaSuccess;
    snappy_decompress_kernel<<<(n_jobs + 7) / 8, 256, 0, st>>>(jobs, n_jobs, status);
    note_launch();
    return cudaGetLastError();
}

__global__ void parquet_level_lengths_kernel(const __grid_constant__ ParquetDecodeParams P) {
    const int p = P.page_lo + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (p >= P.page_hi) return;
    ParquetPage& pg = P.pages[p];
    if (pg.levels >= 0) return;
    const uint8_t* const d = (const uint8_t*)pg.data;
    long long lev = -1;
    if (pg.data_bytes >= 4) lev = (long long)((unsigned)d[0] | (unsigned)d[1] << 8 | (unsigned)d[2] << 16 | (unsigned)d[3] << 24);
    if (lev < 0 || 4 + lev > pg.data_bytes) {
        atomicAdd(P.status, 1ull);
        pg.levels = 0;  // the later kernels then find nothing to read
        pg.values_off = pg.data_bytes;
    } else {
        pg.levels = (int32_t)lev;
        pg.values_off = 4 + (int32_t)lev;
    }
}

cudaError_t launch_parquet_level_lengths(const ParquetDecodeParams& p, cudaStream_t st) {
    if (p.page_hi <= p.page_lo) return cudaSuccess;
    parquet_level_lengths_kernel<<<(p.page_hi - p.page_lo + 255) / 256, 256, 0, st>>>(p);
    note_launch();
    return cudaGetLastError();
}

// One block per job: bytes [src, src + bytes) to dst (16-byte loads and stores where both sides
// share an alignment, single bytes otherwise).
__global__ void __launch_bounds__(256) copy_jobs_kernel(const CopyJob* __restrict__ jobs, int32_t n_jobs) {
    const CopyJob j = jobs[blockIdx.x];
    const uintptr_t s = (uintptr_t)j.src, d = (uintptr_t)j.dst;
    if (((s ^ d) & 15) == 0) {
        const int64_t lead = (int64_t)((16 - (s & 15)) & 15);
        const int64_t head = j.bytes < lead ? j.bytes : lead;
        for (int64_t i = threadIdx.x; i < head; i += blockDim.x) j.dst[i] = j.src[i];
        const int64_t nv = (j.bytes - head) >> 4;
        const uint4* sv = reinterpret_cast<const uint4*>(j.src + head);
        uint4* dv = reinterpret_cast<uint4*>(j.dst + head);
        for (int64_t i = threadIdx.x; i < nv; i += blockDim.x) dv[i] = sv[i];
        for (int64_t i = head + nv * 16 + threadIdx.x; i < j.bytes; i += blockDim.x) j.dst[i] = j.src[i];
    } else {
        for (int64_t i = threadIdx.x; i < j.bytes; i += blockDim.x) j.dst[i] = j.src[i];
    }
}

cudaError_t launch_copy_jobs(const CopyJob* jobs, int32_t n_jobs, cudaStream_t st) {
    if (n_jobs <= 0) return cudaSuccess;
    copy_jobs_kernel<<<n_jobs, 256, 0, st>>>(jobs, n_jobs);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_parquet_levels(const ParquetDecodeParams& p, cudaStream_t st) {
    if (p.page_hi <= p.page_lo) return cudaSuccess;
    parquet_levels_kernel<<<p.page_hi - p.page_lo, 256, 0, st>>>(p);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_parquet_values(const ParquetDecodeParams& p, cudaStream_t st) {
    if (p.item_hi <= p.item_lo) return cudaSuccess;
    parquet_values_kernel<<<p.item_hi - p.item_lo, 256, 0, st>>>(p);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_category_remap(int32_t* codes, int64_t n, const int32_t* table, int32_t table_n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 152 * 8));
    category_remap_kernel<<<(int)blocks, threads, 0, st>>>(codes, n, table, table_n);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_category_insert(int32_t* codes, int64_t n, int32_t pos, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 152 * 8));
    category_insert_kernel<<<(int)blocks, threads, 0, st>>>(codes, n, pos);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_gather_columns(const GatherColumnsParams& p, cudaStream_t st) {
    if (p.n_out <= 0 || p.num_columns <= 0) return cudaSuccess;
    int dev = 0, sms = 1, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gather_columns_kernel, 256, 0);
    if (per_sm < 1) per_sm = 1;
    const int64_t steps = (p.n_out + 32 * kGatherRowsPerLane - 1) / (32 * kGatherRowsPerLane);
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>((steps + 7) / 8, (int64_t)sms * per_sm));
    gather_columns_kernel<<<(int)grid, 256, 0, st>>>(p);
    note_launch();
    return cudaGetLastError();
}

}  // namespace ral
