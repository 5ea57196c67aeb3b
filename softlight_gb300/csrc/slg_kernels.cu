/*
 * slg_kernels.cu - the draw-path kernels that run no shader program: the
 * tile scan, the tile lists, the per-tile key sort of the ordered raster,
 * clears, blits, uniform-block uploads and the scene-graph producer, and the
 * launch sequence that joins them with a program set's vertex and raster
 * stages (slg_pipeline.cuh).
 */
#include "slg_pipeline.cuh"
#include "slg_kernels.cuh"

namespace slg
{

/*-----------------------------------------------------------------------------
 * Kernel 2: exclusive scan of tile counts (one CTA)
-----------------------------------------------------------------------------*/
__global__ void __launch_bounds__(1024) tile_scan_kernel(const Frame f, int numTiles)
{
    __shared__ uint32_t sWarp[32];
    __shared__ uint32_t sCarry;
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    if (tid == 0) sCarry = 0;
    __syncthreads();

    /* 4096 tiles per step: four consecutive tiles per thread (one 16-byte
     * load where the arrays allow it), warp-shuffle scan of the thread sums,
     * warp sums scanned by warp 0 */
    const bool vec = ((reinterpret_cast<uintptr_t>(f.tileCount) | reinterpret_cast<uintptr_t>(f.tileOffset) |
                       reinterpret_cast<uintptr_t>(f.tileCursor)) & 15u) == 0;
    uint32_t c[4] = {0u, 0u, 0u, 0u};
    for (int base = 0; base < numTiles; base += 4096)
    {
        const int t0 = base + 4 * tid;
        if (vec && t0 + 3 < numTiles)
        {
            const uint4 q = *reinterpret_cast<const uint4*>(f.tileCount + t0);
            c[0] = q.x; c[1] = q.y; c[2] = q.z; c[3] = q.w;
        }
        else
        {
#pragma unroll
            for (int k = 0; k < 4; ++k) c[k] = (t0 + k < numTiles) ? f.tileCount[t0 + k] : 0u;
        }
        const uint32_t p1 = c[0], p2 = p1 + c[1], p3 = p2 + c[2], sum = p3 + c[3];
        uint32_t v = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, v, o);
            if (lane >= o) v += n;
        }
        if (lane == 31) sWarp[warp] = v;
        __syncthreads();
        if (warp == 0)
        {
            uint32_t w = sWarp[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, w, o);
                if (lane >= o) w += n;
            }
            sWarp[lane] = w;
        }
        __syncthreads();
        const uint32_t carry = sCarry;
        const uint32_t excl = carry + (warp ? sWarp[warp - 1] : 0u) + v - sum;
        const uint32_t off[4] = {excl, excl + p1, excl + p2, excl + p3};
        if (vec && t0 + 3 < numTiles)
        {
            const uint4 o4 = make_uint4(off[0], off[1], off[2], off[3]);
            *reinterpret_cast<uint4*>(f.tileOffset + t0) = o4;
            *reinterpret_cast<uint4*>(f.tileCursor + t0) = o4;
            *reinterpret_cast<uint4*>(f.tileCount + t0) = make_uint4(0u, 0u, 0u, 0u);
        }
        else
        {
#pragma unroll
            for (int k = 0; k < 4; ++k)
            {
                if (t0 + k < numTiles)
                {
                    f.tileOffset[t0 + k] = off[k];
                    f.tileCursor[t0 + k] = off[k];
                    f.tileCount[t0 + k] = 0;
                }
            }
        }
        __syncthreads();
        if (tid == 1023) sCarry = carry + sWarp[31];
        __syncthreads();
    }
    if (tid == 0)
    {
        const uint32_t total = sCarry;
        f.tileOffset[numTiles] = total;
        if (total > f.entryCap)
        {
            atomicOr(f.status, kStatusEntryOverflow);
            atomicMax(f.status + 1, (int)min(total, 0x7FFFFFFFu));
        }
        *f.ovfCount = 0;
        *f.clipCount = 0;
    }
    if (f.tileOrder != nullptr && numTiles <= 4096)
    {
        /* the ordered raster's tile order: longest list first, by a counting
         * sort of the counts (c: this thread's four tiles, the loop's only
         * step) into 256 buckets scaled to the longest list; the order
         * within a bucket is the atomics' */
        __shared__ uint32_t sHist[256];
        __shared__ uint32_t sMax;
        if (tid == 0) sMax = 0;
        if (tid < 256) sHist[tid] = 0;
        __syncthreads();
        uint32_t m = max(max(c[0], c[1]), max(c[2], c[3]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
        if (lane == 0) atomicMax(&sMax, m);
        __syncthreads();
        const uint64_t maxN = sMax;
        uint32_t b[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            b[k] = maxN ? (uint32_t)(((maxN - c[k]) * 255u) / maxN) : 0u;
            if (4 * tid + k < numTiles) atomicAdd(&sHist[b[k]], 1u);
        }
        __syncthreads();
        if (tid == 0)
        {
            uint32_t run = 0;
            for (int i = 0; i < 256; ++i)
            {
                const uint32_t h = sHist[i];
                sHist[i] = run;
                run += h;
            }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            if (4 * tid + k < numTiles) f.tileOrder[atomicAdd(&sHist[b[k]], 1u)] = (uint32_t)(4 * tid + k);
        }
    }
}

/*-----------------------------------------------------------------------------
 * Kernel 3: tile list fill
-----------------------------------------------------------------------------*/
__device__ __forceinline__ void fill_record(const Frame& f, uint64_t recIndex, uint32_t key)
{
    const float4 r6 = f.records[recIndex * kRecordVec4 + 6];
    const TileRange t = tile_range(r6, f);
    for (int ty = t.ty0; ty <= t.ty1; ++ty)
    {
        for (int tx = t.tx0; tx <= t.tx1; ++tx)
        {
            const uint32_t pos = atomicAdd(&f.tileCursor[ty * f.tilesX + tx], 1u);
            if (pos < f.entryCap)
            {
                f.entries[pos] = key;
            }
        }
    }
}

__global__ void __launch_bounds__(256) bin_fill_kernel(const Frame f)
{
    const uint64_t slot = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t info = (slot < f.numSlots) ? f.slotInfo[slot] : 0u;
    TileRange tr;
    tr.tx0 = 0; tr.tx1 = -1; tr.ty0 = 0; tr.ty1 = -1;
    if (info == 1)
    {
        tr = tile_range(f.records[slot * kRecordVec4 + 6], f);
    }
    /* the ordering key: slot << 3 | sub, or the record's rank in a launch
     * whose order flush_sort_kernel computed */
    const uint32_t key = f.rankOf ? ((info == 1) ? f.rankOf[slot] : 0u) : (uint32_t)(slot << kSubShift);
    warp_tile_walk(f, tr, info == 1, f.tileCursor, [&](uint32_t, uint32_t pos) {
        if (pos < f.entryCap) f.entries[pos] = key;
    });
    if (info >= 2)
    {
        const uint32_t base = f.slotOvf[slot];
        for (uint32_t s = 0; s < info - 2; ++s)
        {
            const uint64_t rec = f.numSlots + base + s;
            fill_record(f, rec, f.rankOf ? f.rankOf[rec] : (key | (s + 1)));
        }
    }
}

/*-----------------------------------------------------------------------------
 * Blend order of a multi-mesh draw. With blending, SL_VertexProcessor::
 * flush_rasterizer (softlight/src/SL_VertexProcessor.cpp:84-181) stable-sorts
 * each group of SL_SHADER_MAX_BINNED_PRIMS (1024) consecutive bins by
 * primIndex before rasterising it. primIndex is a triangle's element index
 * within its mesh (softlight/src/SL_TriProcessor.cpp:546-547,626-630), so
 * in a draw_multiple over several meshes the sort interleaves the meshes.
 * Here the bins are numbered in push order (a scan of the per-slot bin
 * counts), each group is sorted by (primIndex, position in the group), and
 * the tile lists hold each record's rank in that order.
-----------------------------------------------------------------------------*/
constexpr int kFlushGroup = 1024;   /* SL_SHADER_MAX_BINNED_PRIMS */
constexpr int kBinBlock = 1024;     /* slots per block of the bin numbering */

__device__ __forceinline__ uint32_t slot_bins(uint32_t info) { return (info == 1) ? 1u : (info >= 2 ? info - 2u : 0u); }

/* Block-wide exclusive scan of one value per thread (1024 threads); returns
 * the thread's exclusive prefix and sets total. */
__device__ __forceinline__ uint32_t block_scan_1024(uint32_t v, uint32_t* sWarp, uint32_t& total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += n;
    }
    if (lane == 31) sWarp[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
        uint32_t w = sWarp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= o) w += n;
        }
        sWarp[lane] = w;
    }
    __syncthreads();
    total = sWarp[31];
    const uint32_t excl = (warp ? sWarp[warp - 1] : 0u) + incl - v;
    __syncthreads();
    return excl;
}

/* bins per block of 1024 slots */
__global__ void __launch_bounds__(kBinBlock) bin_block_sums_kernel(const Frame f)
{
    __shared__ uint32_t sWarp[32];
    const uint64_t slot = (uint64_t)blockIdx.x * kBinBlock + threadIdx.x;
    const uint32_t b = (slot < f.numSlots) ? slot_bins(f.slotInfo[slot]) : 0u;
    uint32_t total;
    (void)block_scan_1024(b, sWarp, total);
    if (threadIdx.x == 0) f.binBlocks[blockIdx.x] = total;
}

/* exclusive scan of the block sums in place (one CTA); [numBlocks] = total */
__global__ void __launch_bounds__(1024) bin_block_scan_kernel(const Frame f, uint32_t numBlocks)
{
    __shared__ uint32_t sWarp[32];
    uint32_t carry = 0;
    for (uint32_t base = 0; base < numBlocks; base += 1024)
    {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = (i < numBlocks) ? f.binBlocks[i] : 0u;
        uint32_t total;
        const uint32_t excl = block_scan_1024(v, sWarp, total);
        if (i < numBlocks) f.binBlocks[i] = carry + excl;
        carry += total;
    }
    if (threadIdx.x == 0) f.binBlocks[numBlocks] = carry;
}

__device__ __forceinline__ unsigned long long record_prim_index(const Frame& f, uint64_t rec)
{
    const float4 r7 = f.records[rec * kRecordVec4 + 7];
    return ((unsigned long long)__float_as_uint(r7.z) << 32) | __float_as_uint(r7.y);
}

/* every bin's record and primIndex at its push-order number */
__global__ void __launch_bounds__(kBinBlock) bin_seq_kernel(const Frame f)
{
    __shared__ uint32_t sWarp[32];
    const uint64_t slot = (uint64_t)blockIdx.x * kBinBlock + threadIdx.x;
    const uint32_t info = (slot < f.numSlots) ? f.slotInfo[slot] : 0u;
    uint32_t total;
    const uint32_t seq = f.binBlocks[blockIdx.x] + block_scan_1024(slot_bins(info), sWarp, total);
    const uint32_t key = (uint32_t)(slot << kSubShift);
    if (info == 1)
    {
        f.seqRec[seq] = (uint32_t)slot;
        if (f.rankOf) f.seqKey[seq] = record_prim_index(f, slot);
        if (f.itemKey) f.itemKey[seq] = key;
    }
    else if (info >= 2)
    {
        /* the clipped fan's records, in the reference's push order */
        const uint32_t base = f.slotOvf[slot];
        for (uint32_t s = 0; s < info - 2; ++s)
        {
            const uint64_t rec = f.numSlots + base + s;
            f.seqRec[seq + s] = (uint32_t)rec;
            if (f.rankOf) f.seqKey[seq + s] = record_prim_index(f, rec);
            if (f.itemKey) f.itemKey[seq + s] = key | (s + 1);
        }
    }
}

/* One CTA per group of 1024 bins (grid-stride over the groups): stable sort
 * by primIndex, i.e. by (primIndex, position), then each record's rank. */
__global__ void __launch_bounds__(1024) flush_sort_kernel(const Frame f, uint32_t numBlocks)
{
    __shared__ unsigned long long sKey[kFlushGroup];
    const uint32_t total = f.binBlocks[numBlocks];
    for (uint32_t g0 = blockIdx.x * kFlushGroup; g0 < total; g0 += gridDim.x * kFlushGroup)
    {
        const uint32_t n = min((uint32_t)kFlushGroup, total - g0);
        for (uint32_t i = threadIdx.x; i < kFlushGroup; i += blockDim.x)
        {
            sKey[i] = (i < n) ? ((f.seqKey[g0 + i] << 10) | i) : ~0ull;
        }
        __syncthreads();
        for (int k = 2; k <= kFlushGroup; k <<= 1)
        {
            for (int j = k >> 1; j > 0; j >>= 1)
            {
                for (int i = threadIdx.x; i < kFlushGroup; i += blockDim.x)
                {
                    const int ixj = i ^ j;
                    if (ixj > i)
                    {
                        const unsigned long long a = sKey[i], b = sKey[ixj];
                        if ((a > b) == ((i & k) == 0))
                        {
                            sKey[i] = b;
                            sKey[ixj] = a;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (uint32_t p = threadIdx.x; p < n; p += blockDim.x)
        {
            const uint32_t rec = f.seqRec[g0 + (uint32_t)(sKey[p] & (kFlushGroup - 1))];
            f.rankOf[rec] = g0 + p;
            f.recOfRank[g0 + p] = rec;
        }
        __syncthreads();
    }
}

/*-----------------------------------------------------------------------------
 * Tile lists in key order for the ordered raster. The bins, taken in key
 * order (push order, or rank order when flush_sort_kernel ranked them), are
 * cut into binChunks equal runs, one warp each. A counting pass gives every
 * (tile, chunk) its entries, a scan over the chunks of each tile gives the
 * chunk's first position in the tile's list, and the fill pass writes each
 * chunk's entries there in key order. Both passes expand 32 consecutive bins
 * at a time into their (bin, tile) entries, in bin order, and deal the
 * entries to the lanes 32 at a time; lanes holding the same tile are grouped
 * with __match_any_sync, so a tile's entries of one step take consecutive
 * positions in lane (= key) order and one lane advances the chunk's cursor.
 * The lists come out sorted, with no atomics on shared tile cursors and no
 * tile sort.
-----------------------------------------------------------------------------*/
constexpr int kOrderedWarps = 4;   /* chunks (warps) per CTA of the count and fill passes */

__device__ __forceinline__ void bin_item(const Frame& f, uint32_t i, uint32_t& rec, uint32_t& key)
{
    if (f.recOfRank)
    {
        rec = f.recOfRank[i];
        key = i;
    }
    else
    {
        rec = f.seqRec[i];
        key = f.itemKey[i];
    }
}

/* bins [begin, end) of a chunk: equal runs, a multiple of 32 long */
__device__ __forceinline__ void chunk_bins(const Frame& f, uint32_t numBlocks, uint32_t chunk, uint32_t& begin, uint32_t& end)
{
    const uint32_t total = f.binBlocks[numBlocks];
    const uint32_t per = (((total + f.binChunks - 1) / f.binChunks) + 31u) & ~31u;
    begin = min(chunk * per, total);
    end = min(begin + per, total);
}

struct GroupBins
{
    uint32_t start[32];     /* first entry of each bin of the group (exclusive scan) */
    int4 range[32];         /* (tx0, width, ty0, unused) */
    uint32_t key[32];
};

/* Walks the (bin, tile) entries of the chunk's bins in order, 32 per step;
 * fn(tile, key, peers, valid) runs on every lane of every step (peers: the
 * lanes of the step holding the same tile). Every lane of the warp calls it. */
template <class Fn>
__device__ __forceinline__ void for_chunk_entries(const Frame& f, uint32_t begin, uint32_t end, GroupBins& g, Fn&& fn)
{
    const int lane = threadIdx.x & 31;
    for (uint32_t g0 = begin; g0 < end; g0 += 32)
    {
        const uint32_t i = g0 + lane;
        uint32_t n = 0;
        int4 rg = make_int4(0, 1, 0, 0);
        uint32_t key = 0;
        if (i < end)
        {
            uint32_t rec;
            bin_item(f, i, rec, key);
            const TileRange t = tile_range(f.records[(size_t)rec * kRecordVec4 + 6], f);
            if (t.tx1 >= t.tx0 && t.ty1 >= t.ty0)
            {
                rg = make_int4(t.tx0, t.tx1 - t.tx0 + 1, t.ty0, 0);
                n = (uint32_t)rg.y * (uint32_t)(t.ty1 - t.ty0 + 1);
            }
        }
        uint32_t incl = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += v;
        }
        const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
        __syncwarp();
        g.start[lane] = incl - n;
        g.range[lane] = rg;
        g.key[lane] = key;
        __syncwarp();
        for (uint32_t e0 = 0; e0 < total; e0 += 32)
        {
            const uint32_t e = e0 + lane;
            const bool valid = e < total;
            uint32_t tile = 0xFFFFFFFFu, k = 0;
            if (valid)
            {
                /* the bin holding entry e: the last one starting at or before e
                 * (empty bins share their start with the next one) */
                int lo = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1)
                {
                    if (lo + step < 32 && g.start[lo + step] <= e) lo += step;
                }
                const int4 r = g.range[lo];
                const uint32_t local = e - g.start[lo];
                const uint32_t w = (uint32_t)r.y;
                tile = (uint32_t)((r.z + (int)(local / w)) * f.tilesX + r.x + (int)(local % w));
                k = g.key[lo];
            }
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, tile);
            fn(tile, k, peers, valid);
            __syncwarp();
        }
    }
}

/* Per chunk, its entries per tile: a histogram in the warp's shared memory,
 * then one coalesced row of the chunk-major count matrix. */
__global__ void __launch_bounds__(kOrderedWarps * 32) bin_count_ordered_kernel(const Frame f, uint32_t numBlocks)
{
    __shared__ GroupBins sGroup[kOrderedWarps];
    extern __shared__ uint32_t sHist[];   /* [kOrderedWarps][numTiles] */
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t chunk = blockIdx.x * kOrderedWarps + warp;
    if (chunk >= f.binChunks || (f.status[0] & kStatusSticky))
    {
        return;
    }
    const uint32_t numTiles = (uint32_t)(f.tilesX * f.tilesY);
    uint32_t* h = sHist + (size_t)warp * numTiles;
    for (uint32_t t = lane; t < numTiles; t += 32) h[t] = 0u;
    __syncwarp();
    uint32_t begin, end;
    chunk_bins(f, numBlocks, chunk, begin, end);
    for_chunk_entries(f, begin, end, sGroup[warp], [&](uint32_t tile, uint32_t, uint32_t peers, bool valid) {
        /* one lane per tile of the step; steps are separated by __syncwarp */
        if (valid && lane == __ffs(peers) - 1) h[tile] += (uint32_t)__popc(peers);
    });
    __syncwarp();
    uint32_t* row = f.chunkCounts + (size_t)chunk * numTiles;
    for (uint32_t t = lane; t < numTiles; t += 32) row[t] = h[t];
}

/* 32 tiles per CTA, one per lane; warp w scans chunks [w * per, (w+1) * per)
 * of the chunk-major matrix (coalesced rows), the warps' sums are scanned in
 * shared memory, and every count becomes the chunk's first position in the
 * tile's list (relative); each tile's total goes to tileCount. */
__global__ void __launch_bounds__(1024) bin_chunk_scan_kernel(const Frame f)
{
    __shared__ uint32_t sSum[32][33];
    if (f.status[0] & kStatusSticky)
    {
        return;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t numTiles = (uint32_t)(f.tilesX * f.tilesY);
    const uint32_t t = blockIdx.x * 32 + lane;
    const uint32_t W = f.binChunks;
    const uint32_t per = (W + 31) / 32;
    const uint32_t c0 = min(warp * per, W), c1 = min(c0 + per, W);
    uint32_t sum = 0;
    if (t < numTiles)
    {
        for (uint32_t c = c0; c < c1; ++c) sum += f.chunkCounts[(size_t)c * numTiles + t];
    }
    sSum[warp][lane] = sum;
    __syncthreads();
    uint32_t base = 0;
    for (int w = 0; w < warp; ++w) base += sSum[w][lane];
    if (t < numTiles)
    {
        for (uint32_t c = c0; c < c1; ++c)
        {
            uint32_t* p = f.chunkCounts + (size_t)c * numTiles + t;
            const uint32_t v = *p;
            *p = base;
            base += v;
        }
        if (warp == 31) f.tileCount[t] = base;
    }
}

/* Each chunk's entries at its cursors: the warp's cursors (tile list offset
 * + the chunk's first position) live in its shared memory. */
__global__ void __launch_bounds__(kOrderedWarps * 32) bin_fill_ordered_kernel(const Frame f, uint32_t numBlocks)
{
    __shared__ GroupBins sGroup[kOrderedWarps];
    extern __shared__ uint32_t sCursor[];   /* [kOrderedWarps][numTiles] */
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t chunk = blockIdx.x * kOrderedWarps + warp;
    if (chunk >= f.binChunks || (f.status[0] & kStatusSticky))
    {
        return;
    }
    const uint32_t numTiles = (uint32_t)(f.tilesX * f.tilesY);
    uint32_t* cur = sCursor + (size_t)warp * numTiles;
    const uint32_t* row = f.chunkCounts + (size_t)chunk * numTiles;
    for (uint32_t t = lane; t < numTiles; t += 32) cur[t] = f.tileOffset[t] + row[t];
    __syncwarp();
    uint32_t begin, end;
    chunk_bins(f, numBlocks, chunk, begin, end);
    for_chunk_entries(f, begin, end, sGroup[warp], [&](uint32_t tile, uint32_t key, uint32_t peers, bool valid) {
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (valid && lane == leader) base = cur[tile];
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        if (valid)
        {
            const uint32_t pos = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
            if (pos < f.entryCap) f.entries[pos] = key;
            /* the step's entries of this tile advance the chunk's cursor */
            if (lane == leader) cur[tile] = base + (uint32_t)__popc(peers);
        }
    });
}

/*-----------------------------------------------------------------------------
 * Tile sort of the ordered raster
-----------------------------------------------------------------------------*/
/* Sorts each tile's key list in place (ascending = submission order) for
 * the ordered raster; one CTA per tile, the list staged in shared memory. */
__global__ void __launch_bounds__(1024) tile_sort_kernel(const Frame f, int sortCap)
{
    extern __shared__ __align__(16) uint8_t smem[];
    uint32_t* sKeys = reinterpret_cast<uint32_t*>(smem);
    const int tile = blockIdx.x;
    const uint32_t begin = f.tileOffset[tile];
    const uint32_t n = f.tileOffset[tile + 1] - begin;
    if (n < 2 || (f.status[0] & kStatusSticky) || !ordered_raster_runs(f))
    {
        return;
    }
    if ((int)n > sortCap)
    {
        if (!f.sortScratch)
        {
            if (threadIdx.x == 0) atomicOr(f.status, kStatusTileOverflow);
            return;
        }
        /* bitonic sort in global memory: the list padded to p <= 2n keys at
         * twice its offset, so the tiles' regions never overlap */
        uint32_t* g = f.sortScratch + 2ull * begin;
        uint32_t p = 2;
        while (p < n) p <<= 1;
        for (uint32_t i = threadIdx.x; i < p; i += blockDim.x) g[i] = (i < n) ? f.entries[begin + i] : 0xFFFFFFFFu;
        __syncthreads();
        for (uint32_t k = 2; k <= p; k <<= 1)
        {
            for (uint32_t j = k >> 1; j > 0; j >>= 1)
            {
                for (uint32_t i = threadIdx.x; i < p; i += blockDim.x)
                {
                    const uint32_t ixj = i ^ j;
                    if (ixj > i)
                    {
                        const uint32_t a = g[i], b = g[ixj];
                        if ((a > b) == ((i & k) == 0))
                        {
                            g[i] = b;
                            g[ixj] = a;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) f.entries[begin + i] = g[i];
        return;
    }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) sKeys[i] = f.entries[begin + i];
    __syncthreads();
    sort_keys(sKeys, (int)n);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) f.entries[begin + i] = sKeys[i];
}

/* kGeneral: the instantiation that carries line and wireframe records and
 * writes several render targets (such launches use kLineTile tiles); the
/*-----------------------------------------------------------------------------
 * Clear (SL_ClearProcessor, softlight/src/SL_ClearProcessor.cpp)
-----------------------------------------------------------------------------*/
struct TexelValue { uint32_t w[8]; };   /* up to 32 bytes of one texel */

__global__ void clear_kernel(uint8_t* dst, size_t numTexels, int bytesPerTexel, TexelValue value, const int32_t* status)
{
    if (status && (*status & kStatusSticky))
    {
        return;   /* replayed once the launch that overflowed has been */
    }
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < numTexels; i += stride)
    {
        if (bytesPerTexel == 16) reinterpret_cast<uint4*>(dst)[i] = make_uint4(value.w[0], value.w[1], value.w[2], value.w[3]);
        else if (bytesPerTexel == 8) reinterpret_cast<uint2*>(dst)[i] = make_uint2(value.w[0], value.w[1]);
        else if (bytesPerTexel == 4) reinterpret_cast<uint32_t*>(dst)[i] = value.w[0];
        else if (bytesPerTexel == 2) reinterpret_cast<uint16_t*>(dst)[i] = (uint16_t)value.w[0];
        else
        {
            /* 1, 3, 6, 12, 24 or 32 bytes: byte by byte */
            const uint8_t* v = reinterpret_cast<const uint8_t*>(value.w);
            for (int b = 0; b < bytesPerTexel; ++b) dst[i * (size_t)bytesPerTexel + b] = v[b];
        }
    }
}

/*-----------------------------------------------------------------------------
 * Scene graph: SL_SceneGraph::update (softlight/src/SL_SceneGraph.cpp:223-299)
 * and the draw list of a mesh-node traversal, in the arithmetic of the
 * LightMath layer the reference sources are built against (mat4 * vec4 sums
 * the scaled columns left to right; mat4 * mat4 applies that per column).
-----------------------------------------------------------------------------*/
struct M4
{
    float4 c[4];
};

__device__ __forceinline__ float4 m4_apply(const M4& a, const float4 v)
{
    return make_float4(((a.c[0].x * v.x + a.c[1].x * v.y) + a.c[2].x * v.z) + a.c[3].x * v.w,
                       ((a.c[0].y * v.x + a.c[1].y * v.y) + a.c[2].y * v.z) + a.c[3].y * v.w,
                       ((a.c[0].z * v.x + a.c[1].z * v.y) + a.c[2].z * v.z) + a.c[3].z * v.w,
                       ((a.c[0].w * v.x + a.c[1].w * v.y) + a.c[2].w * v.z) + a.c[3].w * v.w);
}

__device__ __forceinline__ M4 m4_mul(const M4& a, const M4& b)
{
    M4 r;
#pragma unroll
    for (int i = 0; i < 4; ++i) r.c[i] = m4_apply(a, b.c[i]);
    return r;
}

__device__ __forceinline__ M4 m4_load(const float* p)
{
    M4 r;
#pragma unroll
    for (int i = 0; i < 4; ++i) r.c[i] = make_float4(p[4 * i], p[4 * i + 1], p[4 * i + 2], p[4 * i + 3]);
    return r;
}

__device__ __forceinline__ void m4_store(float* p, const M4& m)
{
#pragma unroll
    for (int i = 0; i < 4; ++i)
    {
        p[4 * i] = m.c[i].x;
        p[4 * i + 1] = m.c[i].y;
        p[4 * i + 2] = m.c[i].z;
        p[4 * i + 3] = m.c[i].w;
    }
}

/* SL_Transform::get_rst_matrix / get_str_matrix (softlight/src/SL_Transform.cpp:
 * 408-432): (translation x scale) * R or R * (translation x scale), R the
 * rotation of the orientation quaternion (columns (1-2(yy+zz), 2(xy+wz),
 * 2(xz-wy)), (2(xy-wz), 1-2(xx+zz), 2(yz+wx)), (2(xz+wy), 2(yz-wx),
 * 1-2(xx+yy))). */
__device__ M4 scene_local(const SceneNodeGpu& n)
{
    const float x = n.orientation[0], y = n.orientation[1], z = n.orientation[2], w = n.orientation[3];
    const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z, wx = w * x, wy = w * y, wz = w * z;
    M4 r;
    r.c[0] = make_float4(1.f - 2.f * (yy + zz), 2.f * (xy + wz), 2.f * (xz - wy), 0.f);
    r.c[1] = make_float4(2.f * (xy - wz), 1.f - 2.f * (xx + zz), 2.f * (yz + wx), 0.f);
    r.c[2] = make_float4(2.f * (xz + wy), 2.f * (yz - wx), 1.f - 2.f * (xx + yy), 0.f);
    r.c[3] = make_float4(0.f, 0.f, 0.f, 1.f);
    M4 ts;
    ts.c[0] = make_float4(n.scaling[0], 0.f, 0.f, 0.f);
    ts.c[1] = make_float4(0.f, n.scaling[1], 0.f, 0.f);
    ts.c[2] = make_float4(0.f, 0.f, n.scaling[2], 0.f);
    ts.c[3] = make_float4(n.position[0], n.position[1], n.position[2], 1.f);
    return n.viewFps ? m4_mul(r, ts) : m4_mul(ts, r);
}

/* One thread per recomputed node: update_node_transform sets
 * model = parent's model * local (apply_pre_transform), or local for a node
 * of the root. The parent's model is the one this update computes when the
 * parent is recomputed too (it precedes the node in the reference's loop),
 * so the thread walks up through recomputed ancestors and multiplies down;
 * every thread writes only its own node. */
__global__ void __launch_bounds__(128) scene_update_kernel(const SceneNodeGpu* nodes, const uint32_t* list, uint32_t n, float* model)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
    {
        return;
    }
    uint32_t chain[kSceneMaxDepth];
    int len = 0;
    uint64_t c = list[i];
    for (;;)
    {
        chain[len++] = (uint32_t)c;
        const uint64_t p = nodes[c].parent;
        if (p == kSceneRoot || !nodes[p].update || len == kSceneMaxDepth)
        {
            break;
        }
        c = p;
    }
    const uint64_t top = chain[len - 1];
    const uint64_t topParent = nodes[top].parent;
    M4 m = scene_local(nodes[top]);
    if (topParent != kSceneRoot)
    {
        m = m4_mul(m4_load(model + 16 * topParent), m);
    }
    for (int k = len - 2; k >= 0; --k)
    {
        m = m4_mul(m, scene_local(nodes[chain[k]]));
    }
    m4_store(model + 16 * (uint64_t)list[i], m);
}

/* One thread per draw of the list: the traversal of SoftLight's scene demos
 * (softlight/tests/sl_large_scene_test.cpp:689-740): mv = view * model,
 * sl_is_visible(bounds, mv, frustum planes) (softlight/src/SL_Camera.cpp:
 * 63-85), then the draw's uniform block. */
__global__ void __launch_bounds__(128) scene_draw_kernel(const SceneDrawArgs a)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.numEntries)
    {
        return;
    }
    const SceneEntryGpu en = a.entries[e];
    const float* mp = a.model + 16 * en.node;
    bool visible = true;
    if (a.cull)
    {
        const M4 mv = m4_mul(m4_load(a.view), m4_load(mp));
        const float* b = a.bounds + 8 * (uint64_t)en.bounds;
        const float4 bmax = m4_apply(mv, make_float4(b[0], b[1], b[2], b[3]));
        const float4 bmin = m4_apply(mv, make_float4(b[4], b[5], b[6], b[7]));
        const float cx = (bmax.x + bmin.x) * 0.5f, cy = (bmax.y + bmin.y) * 0.5f, cz = (bmax.z + bmin.z) * 0.5f;
        const float hx = (bmax.x - bmin.x) * 0.5f, hy = (bmax.y - bmin.y) * 0.5f, hz = (bmax.z - bmin.z) * 0.5f;
        const float radius = sqrtf((hx * hx + hy * hy) + hz * hz);
        for (int i = 0; i < 6; ++i)
        {
            const float* pl = a.planes + 4 * i;
            if (((((cx * pl[0] + cy * pl[1]) + cz * pl[2]) + pl[3]) + radius) <= 0.f)
            {
                visible = false;
                break;
            }
        }
    }
    uint32_t* dst = reinterpret_cast<uint32_t*>(en.ubo);
    for (uint32_t k = 0; k < a.templWords; ++k) dst[k] = a.templ[k];
    float* u = reinterpret_cast<float*>(en.ubo);
    for (int k = 0; k < 16; ++k) u[offsetof(slg_lambert_uniforms, vpMatrix) / 4 + k] = a.vp[k];
    for (int k = 0; k < 16; ++k) u[offsetof(slg_lambert_uniforms, modelMatrix) / 4 + k] = mp[k];
    dst[offsetof(slg_lambert_uniforms, textureId) / 4] = en.textureId;
    a.descs[e].hidden = visible ? 0 : 1;
}

__global__ void __launch_bounds__(64) ubo_scatter_kernel(const uint8_t* stage)
{
    const UboCopy c = reinterpret_cast<const UboCopy*>(stage)[blockIdx.x];
    const uint32_t* src = reinterpret_cast<const uint32_t*>(stage + c.src);
    uint32_t* dst = reinterpret_cast<uint32_t*>(c.dst);
    for (uint32_t w = threadIdx.x; w < c.words; w += blockDim.x) dst[w] = src[w];
}

cudaError_t launch_ubo_scatter(const uint8_t* stage, uint32_t n, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    ubo_scatter_kernel<<<n, 64, 0, s>>>(stage);
    return cudaGetLastError();
}

cudaError_t launch_scene_update(const SceneNodeGpu* nodes, const uint32_t* list, uint32_t n, float* model, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    scene_update_kernel<<<(n + 127) / 128, 128, 0, s>>>(nodes, list, n, model);
    return cudaGetLastError();
}

cudaError_t launch_scene_draw(const SceneDrawArgs& a, cudaStream_t s)
{
    if (a.numEntries == 0) return cudaSuccess;
    scene_draw_kernel<<<(a.numEntries + 127) / 128, 128, 0, s>>>(a);
    return cudaGetLastError();
}

/*-----------------------------------------------------------------------------
 * One launch: the program set's vertex stage, the library's tile scan, tile
 * lists and tile sort, the program set's raster stage.
-----------------------------------------------------------------------------*/
/* After the last kernel that can overflow a buffer: counts the launch as
 * done when no overflow has happened yet (status[3]), which tells the host
 * the first launch to replay. */
__global__ void reset_counts_kernel(const Frame f)
{
    *f.ovfCount = 0;
    *f.clipCount = 0;
}

__global__ void launch_mark_kernel(int32_t* status)
{
    if (!(status[0] & kStatusSticky)) status[3] += 1;
}

cudaError_t init_library_attributes(int keyCap)
{
    const int chunkSmem = (int)(sizeof(uint32_t) * kOrderedWarps * kMaxOrderedTiles);
    cudaError_t e = cudaFuncSetAttribute(tile_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(sizeof(uint32_t) * keyCap));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(bin_count_ordered_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, chunkSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(bin_fill_ordered_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, chunkSmem);
    return e;
}

cudaError_t launch_pipeline(const Frame& f, const slg_pipeline_ops& ops, int keyCap, cudaStream_t s, cudaEvent_t* ev)
{
    const int numTiles = f.tilesX * f.tilesY;
    if (ev) cudaEventRecord(ev[0], s);
    if (f.aliasCount)
    {
        cudaMemsetAsync(f.aliasCount, 0, sizeof(uint32_t), s);
    }
    cudaError_t e = (cudaError_t)ops.launch_vertex(&f, s);
    if (e != cudaSuccess) return e;
    const uint32_t numBlocks = (uint32_t)((f.numSlots + kBinBlock - 1) / kBinBlock);
    const bool ordered = f.chunkCounts != nullptr && f.numSlots > 0;
    if ((f.rankOf || ordered) && f.numSlots > 0)
    {
        bin_block_sums_kernel<<<numBlocks, kBinBlock, 0, s>>>(f);
        bin_block_scan_kernel<<<1, 1024, 0, s>>>(f, numBlocks);
        bin_seq_kernel<<<numBlocks, kBinBlock, 0, s>>>(f);
        if (f.rankOf) flush_sort_kernel<<<f.rankGrid, 1024, 0, s>>>(f, numBlocks);
    }
    if (ev) cudaEventRecord(ev[1], s);
    /* the untiled order-free raster needs no tile lists */
    const bool untiled = f.bestWords != nullptr;
    const unsigned chunkBlocks = (f.binChunks + kOrderedWarps - 1) / kOrderedWarps;
    const size_t chunkSmem = sizeof(uint32_t) * kOrderedWarps * (size_t)numTiles;
    if (ordered)
    {
        /* per-chunk counts; their scan also gives each tile's total */
        bin_count_ordered_kernel<<<chunkBlocks, kOrderedWarps * 32, chunkSmem, s>>>(f, numBlocks);
        bin_chunk_scan_kernel<<<(numTiles + 31) / 32, 1024, 0, s>>>(f);
    }
    if (!untiled) tile_scan_kernel<<<1, 1024, 0, s>>>(f, numTiles);
    if (ev) cudaEventRecord(ev[2], s);
    if (ordered)
    {
        bin_fill_ordered_kernel<<<chunkBlocks, kOrderedWarps * 32, chunkSmem, s>>>(f, numBlocks);
    }
    else if (f.numSlots > 0 && !untiled)
    {
        const unsigned blocks = (unsigned)((f.numSlots + 255) / 256);
        bin_fill_kernel<<<blocks, 256, 0, s>>>(f);
    }
    if (ev) cudaEventRecord(ev[3], s);
    if ((!f.orderFree || f.aliasCount) && !ordered && !untiled)
    {
        /* keyCap keys of 4 bytes per tile (<= 227 KB of shared memory); for an
         * order-free launch with line draws the device decides whether the
         * ordered raster runs (ordered_raster_runs) */
        tile_sort_kernel<<<numTiles, 1024, sizeof(uint32_t) * (size_t)keyCap, s>>>(f, keyCap);
    }
    launch_mark_kernel<<<1, 1, 0, s>>>(f.status);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = (cudaError_t)ops.launch_raster(&f, s);
    if (untiled)
    {
        /* the raster read the clipped-record count: reset it (and the clip
         * queue's) for the next launch, as tile_scan_kernel does otherwise */
        reset_counts_kernel<<<1, 1, 0, s>>>(f);
    }
    if (ev) cudaEventRecord(ev[4], s);
    return e;
}

/*-----------------------------------------------------------------------------
 * Blit (SL_BlitProcessor::blit_nearest, softlight/src/SL_BlitProcessor.cpp:621-660,
 * with the blit operators of :20-420 and color_cast of SL_Color.hpp:600-690)
-----------------------------------------------------------------------------*/
__device__ __forceinline__ float4 blit_src_rgbaf(const BlitArgs& a, uint64_t i)
{
    switch (a.srcType)
    {
        case SLG_COLOR_RGBA_8U:
            return unpack_rgba8(reinterpret_cast<const uint32_t*>(a.src)[i]);
        case SLG_COLOR_RGBA_FLOAT:
            return reinterpret_cast<const float4*>(a.src)[i];
        default:
            /* SL_Blit_R_to_RGBA: (min, min, r, max) in the source type */
            return make_float4(0.f, 0.f, reinterpret_cast<const float*>(a.src)[i], 1.f);
    }
}

__global__ void blit_kernel(const BlitArgs a)
{
    if (a.status && (*a.status & kStatusSticky))
    {
        return;   /* replayed once the launch that overflowed has been */
    }
    const uint64_t n = a.nx * a.ny;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride)
    {
        const uint64_t x = a.x0 + t % a.nx;
        const uint64_t y = a.y0 + t / a.nx;
        const uint64_t srcX = (x * a.foutW) >> 16;
        const uint64_t yf = (y * a.foutH) >> 16;
        const uint64_t srcY = a.srcY1 - (a.srcY0 + yf) - 1u;
        const uint64_t si = srcX + a.srcW * srcY;
        const uint64_t di = x + a.dstW * y;
        if (a.srcType == a.dstType)
        {
            /* same format: a plain copy (SL_Blit_RGBA_to_RGBA<u8, u8> copies
             * the 32-bit word; float to float is the identity cast) */
            if (a.dstType == SLG_COLOR_RGBA_FLOAT) reinterpret_cast<float4*>(a.dst)[di] = reinterpret_cast<const float4*>(a.src)[si];
            else reinterpret_cast<uint32_t*>(a.dst)[di] = reinterpret_cast<const uint32_t*>(a.src)[si];
            continue;
        }
        if (a.srcType == SLG_COLOR_RGBA_8U && a.dstType == SLG_COLOR_R_FLOAT)
        {
            /* SL_Blit_RGBA_to_R<uint8_t, float>: the red channel of the cast */
            reinterpret_cast<float*>(a.dst)[di] = (float)(reinterpret_cast<const uint32_t*>(a.src)[si] & 0xFFu) * 0.00392156862745f;
            continue;
        }
        const float4 c = blit_src_rgbaf(a, si);
        switch (a.dstType)
        {
            case SLG_COLOR_RGBA_8U:
            {
                /* color_cast<uint8_t, float>: (uint8_t)(c * 255) per channel */
                const uint32_t r = f2u8(c.x * 255.f), g = f2u8(c.y * 255.f), b = f2u8(c.z * 255.f), w = f2u8(c.w * 255.f);
                reinterpret_cast<uint32_t*>(a.dst)[di] = r | (g << 8) | (b << 16) | (w << 24);
                break;
            }
            case SLG_COLOR_RGBA_FLOAT:
                reinterpret_cast<float4*>(a.dst)[di] = c;
                break;
            default:
                reinterpret_cast<float*>(a.dst)[di] = c.x;
                break;
        }
    }
}

cudaError_t launch_blit(const BlitArgs& a, cudaStream_t s)
{
    const uint64_t n = a.nx * a.ny;
    const unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, 152u * 16u);
    blit_kernel<<<blocks ? blocks : 1, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_clear(uint8_t* dst, size_t numTexels, int bytesPerTexel, const uint32_t value[8], const int32_t* status,
                         cudaStream_t s)
{
    TexelValue v;
    for (int k = 0; k < 8; ++k) v.w[k] = value[k];
    const unsigned blocks = (unsigned)std::min<size_t>((numTexels + 255) / 256, 152u * 16u);
    clear_kernel<<<blocks ? blocks : 1, 256, 0, s>>>(dst, numTexels, bytesPerTexel, v, status);
    return cudaGetLastError();
}

} // namespace slg
