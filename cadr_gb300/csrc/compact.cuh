// compact.cuh - per-StateSet compaction of one tile of drawables.
//
// A tile is THREADS * IPT consecutive drawables; item j of thread t is
// drawable b + j*THREADS + t, so each warp ballot covers 32 consecutive
// drawables and the ballots in (j, warp) order are in drawable order.
// The visible drawables of StateSet s go to cmds[offsets[s] + k] for the
// k-th visible drawable of that region, in ascending drawable order:
//   slot(i) = offsets[s] + (number of visible drawables of region s before i)
// computed as a segmented scan (regions are the segments) whose carry
// between tiles comes from a decoupled lookback over published tile states.
#pragma once

#include "common.cuh"
#include "kernels.cuh"

namespace cadr {

// Segmented decoupled lookback by one warp.  Returns the segmented
// exclusive prefix at the tile start: the number of flagged items from the
// start of the region containing the tile's first item up to that item.
// Lanes inspect 32 predecessors at a time; a predecessor that published its
// inclusive prefix, or whose aggregate contains a region start, ends the
// walk.  Items below `first` count as empty terminators.  Every wait is
// bounded by limit_ns; on expiry timed_out is set and the partial carry
// returned (the pass then reports CADR_ERR_TIMEOUT).
__device__ __forceinline__ uint32_t warp_lookback(const uint64_t* __restrict__ states, int64_t item,
                                                  int64_t first, uint32_t epoch, uint64_t limit_ns,
                                                  bool& timed_out)
{
    const int lane = threadIdx.x & 31;
    const uint32_t ep = epoch & kEpochMask;
    uint32_t carry = 0;
    int64_t cur = item - 1;
    uint64_t t0 = 0;
    for (uint32_t it = 0; it < (1u << 30); it++) {
        const int64_t idx = cur - lane;
        uint64_t w = 0;
        bool valid = true, term = true;
        if (idx >= first) {
            w = load_relaxed_u64(states + idx);
            valid = st_status(w) != 0 && st_epoch(w) == ep;
            term = valid && (st_status(w) == kStatusPrefix || st_head(w));
        }
        const uint32_t tmask = __ballot_sync(~0u, term);
        const uint32_t vmask = __ballot_sync(~0u, valid);
        const int ft = tmask ? __ffs(tmask) - 1 : 32;
        const uint32_t need = (ft >= 31) ? 0xffffffffu : ((2u << ft) - 1u);
        if ((vmask & need) == need) {
            uint32_t v = (lane <= ft && idx >= first) ? st_value(w) : 0u;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(~0u, v, o);
            carry += v;
            if (ft < 32) return carry;
            cur -= 32;
            t0 = 0;
        } else {
            uint64_t now = global_timer_ns();
            now = __shfl_sync(~0u, now, 0);
            if (t0 == 0) {
                t0 = now;
            } else if (now - t0 > limit_ns) {
                timed_out = true;
                return carry;
            }
            __nanosleep(64);
        }
    }
    timed_out = true;
    return carry;
}

template <int THREADS, int IPT>
struct Tile {
    static constexpr int NW = THREADS / kWarp;
    static constexpr int NC = IPT * NW;
    static constexpr int SIZE = THREADS * IPT;
    static_assert(NW >= 2, "two warps at least");

    struct __align__(16) Smem {
        uint32_t ballot[IPT][NW];
        uint32_t prefix[NC];
        uint32_t info[8];  // 0 item, 1 epoch, 2 carry, 3 total, 4 first region, 5 last region,
                           // 6 published value, 7 published head flag
    };

    // Tile-local exclusive prefix of visible items at tile position q (0..SIZE).
    __device__ static __forceinline__ uint32_t excl(const Smem& sm, uint32_t q)
    {
        if (q >= (uint32_t)SIZE) return sm.info[3];
        const uint32_t j = q / THREADS, r = q % THREADS, w = r >> 5, l = r & 31u;
        return sm.prefix[j * NW + w] + __popc(sm.ballot[j][w] & ((1u << l) - 1u));
    }

    // Warp 0: the exclusive prefix of the ballot counts (prefix[]) and the
    // tile's total (info[3]).
    __device__ static __forceinline__ void prefix_warp0(Smem& sm)
    {
        const int lane = threadIdx.x & 31;
        constexpr int PER = (NC + 31) / 32;
        uint32_t c[PER];
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < PER; k++) {
            const int idx = lane * PER + k;
            c[k] = idx < NC ? __popc(sm.ballot[idx / NW][idx % NW]) : 0u;
            sum += c[k];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(~0u, incl, o);
            if (lane >= o) incl += v;
        }
        uint32_t run = incl - sum;
#pragma unroll
        for (int k = 0; k < PER; k++) {
            const int idx = lane * PER + k;
            if (idx < NC) sm.prefix[idx] = run;
            run += c[k];
        }
        if (lane == 31) sm.info[3] = incl;
    }

    // After all ballots are stored and a __syncthreads(): scan the ballot
    // counts (warp 0) and locate the regions of the tile's first and last
    // drawable (warp 1).  Ends with __syncthreads().
    __device__ static __forceinline__ void scan(Smem& sm, const uint32_t* __restrict__ offsets, uint32_t S,
                                                uint32_t b, uint32_t n)
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if (warp == 0) {
            prefix_warp0(sm);
        } else if (warp == 1 && lane == 0) {
            // Clamped to S-1 so that an empty scene (n == 0, one work item)
            // stays inside the offsets and counts arrays.
            const uint32_t e = min(b + (uint32_t)SIZE, n);
            sm.info[4] = min(region_of(offsets, 0, S + 1, b), S - 1);
            sm.info[5] = n ? min(region_of(offsets, 0, S + 1, e - 1), S - 1) : S - 1;
        }
        __syncthreads();
    }

    // scan() for a tile whose regions the caller stored in info[4] and
    // info[5] before the __syncthreads() that precedes it (from the scene's
    // per-tile table): the prefix alone.  Ends with __syncthreads().
    __device__ static __forceinline__ void scan_known_regions(Smem& sm)
    {
        if (threadIdx.x < 32) prefix_warp0(sm);
        __syncthreads();
    }

    // Warp 0 alone, after the ballots are stored and a __syncthreads(): the
    // same results as scan() (ballot-count prefix, total, the regions of
    // the tile's first and last drawable), with no CTA barrier; warp 0 sees
    // them after its own __syncwarp(), the other warps after the caller's
    // next __syncthreads().  The whole warp finds each region in 32-way
    // rounds (the lookback form's tiles need not be the scene table's).
    __device__ static __forceinline__ void scan_warp0(Smem& sm, const uint32_t* __restrict__ offsets, uint32_t S,
                                                      uint32_t b, uint32_t n)
    {
        const int lane = threadIdx.x & 31;
        prefix_warp0(sm);
        // Clamped to S-1 so that an empty scene (n == 0, one work item)
        // stays inside the offsets and counts arrays.
        const uint32_t e = min(b + (uint32_t)SIZE, n);
        const uint32_t rf = min(warp_region_of(offsets, S, b), S - 1);
        const uint32_t rl = n ? min(warp_region_of(offsets, S, e - 1), S - 1) : S - 1;
        if (lane == 0) {
            sm.info[4] = rf;
            sm.info[5] = rl;
        }
        __syncwarp();
    }

    // One lane of warp 0, after scan(): publish the tile's aggregate (the
    // scan's first item publishes its inclusive prefix at once) and keep the
    // published value and head flag in info[6], info[7] for resolve().
    __device__ static __forceinline__ void publish(Smem& sm, uint64_t* __restrict__ states, int64_t item,
                                                   int64_t first, const uint32_t* __restrict__ offsets, uint32_t b,
                                                   uint32_t fault)
    {
        const uint32_t total = sm.info[3];
        const uint32_t last_start = offsets[sm.info[5]];
        const uint32_t head = last_start >= b ? 1u : 0u;
        const uint32_t val = head ? total - excl(sm, last_start - b) : total;
        sm.info[6] = val;
        sm.info[7] = head;
        if (item == first) {
            if (fault != CADR_FAULT_SKIP_FIRST_TILE_PUBLISH)
                store_relaxed_u64(states + item, pack_status(sm.info[1], kStatusPrefix, 1u, val));
        } else {
            store_relaxed_u64(states + item, pack_status(sm.info[1], kStatusAgg, head, val));
        }
    }

    // Warp 0, after publish() and a barrier or in the publishing warp: look
    // back and publish the inclusive prefix; carry in info[2] (visible to the
    // CTA after the caller's next __syncthreads()).
    __device__ static __forceinline__ void resolve(Smem& sm, uint64_t* __restrict__ states, int64_t item,
                                                   int64_t first, uint64_t limit_ns, uint32_t* error)
    {
        const int lane = threadIdx.x & 31;
        __syncwarp();
        uint32_t carry = 0;
        bool timed_out = false;
        if (item != first) {
            const uint32_t epoch = sm.info[1], val = sm.info[6], head = sm.info[7];
            carry = warp_lookback(states, item, first, epoch, limit_ns, timed_out);
            if (lane == 0)
                store_relaxed_u64(states + item, pack_status(epoch, kStatusPrefix, head, head ? val : carry + val));
        }
        if (lane == 0) {
            sm.info[2] = carry;
            if (timed_out) atomicOr(error, CADR_DEVERR_LOOKBACK_TIMEOUT);
        }
    }

    // Every thread: the LOD-table entries of its visible items, all issued
    // together so that their L2 round trips overlap.
    __device__ static __forceinline__ void gather(uint32_t vis_bits, uint32_t lod_bits, const uint32_t (&geo)[IPT],
                                                  const uint4* __restrict__ lods, uint32_t G, uint32_t L,
                                                  uint32_t* error, uint4 (&ent)[IPT])
    {
#pragma unroll
        for (int j = 0; j < IPT; j++) {
            ent[j] = make_uint4(0u, 0u, 0u, 0u);
            if (!((vis_bits >> j) & 1u)) continue;
            uint32_t g = geo[j];
            if (g >= G) {
                atomicOr(error, CADR_DEVERR_BAD_INDEX);
                g = 0;
            }
            ent[j] = __ldg(lods + (size_t)g * L + ((lod_bits >> (2 * j)) & 3u));
        }
    }

    // Every thread: write the commands of its visible items (LOD entries
    // from gather()) and the counts of the regions ending in this tile (the
    // scan's first tile also writes the zero counts of empty regions).
    __device__ static __forceinline__ void write_ent(const Smem& sm, uint32_t vis_bits, const uint4 (&ent)[IPT],
                                                     uint32_t b, uint32_t n, bool first_tile,
                                                     const uint32_t* __restrict__ offsets, uint32_t S,
                                                     uint32_t* __restrict__ cmds, uint32_t* __restrict__ counts,
                                                     uint32_t* error)
    {
        write_cmds<0, IPT>(sm, vis_bits, ent, b, n, offsets, cmds, error);
        write_counts(sm, b, n, first_tile, offsets, S, counts, error);
    }

    // The commands of the thread's visible items in rows [J0, J1); bit j of
    // vis_bits and ent[j - J0] belong to row j.  A slot outside the n
    // commands (only possible from inconsistent offsets or carries) is
    // flagged with CADR_DEVERR_BAD_INDEX and not written.  With kShard the
    // commands are placed by `sp` instead of at offsets[s] + k.
    template <int J0, int J1, bool kShard = false>
    __device__ static __forceinline__ void write_cmds(const Smem& sm, uint32_t vis_bits, const uint4 (&ent)[J1 - J0],
                                                      uint32_t b, uint32_t n, const uint32_t* __restrict__ offsets,
                                                      uint32_t* __restrict__ cmds, uint32_t* error,
                                                      const ShardPlacement& sp = ShardPlacement{})
    {
        const int t = threadIdx.x;
        const uint32_t carry = sm.info[2], rf = sm.info[4], rl = sm.info[5];
        const uint32_t start_f = offsets[rf];
        if (rf == rl) {
            // The whole tile in one region: slot = base + the item's
            // tile-local exclusive prefix (from its row's ballot and prefix).
            const uint32_t lane = (uint32_t)t & 31u, warp = (uint32_t)t >> 5;
            const uint32_t lt = (1u << lane) - 1u;
            const uint32_t base = (start_f >= b) ? start_f - excl(sm, start_f - b) : start_f + carry;
            const uint32_t dbase = kShard ? __ldg(sp.dst_base + rf) : 0u;
#pragma unroll
            for (int j = J0; j < J1; j++) {
                if (!((vis_bits >> j) & 1u)) continue;
                const uint32_t i = b + (uint32_t)(j * THREADS + t);
                const uint32_t slot = base + sm.prefix[j * NW + warp] + __popc(sm.ballot[j][warp] & lt);
                uint32_t out = slot;
                if (kShard) out = (slot < n) ? dbase + (slot - start_f) : 0xffffffffu;
                if (slot >= n || (kShard && out >= sp.capacity)) {
                    atomicOr(error, CADR_DEVERR_BAD_INDEX);
                    continue;
                }
                if (!CADR_CHECKED(in_region(offsets, rf, i, slot), error)) continue;
                const uint4 e = ent[j - J0];
                uint32_t* c = cmds + (size_t)out * 5;
                c[0] = e.x;
                c[1] = 1u;
                c[2] = e.y;
                c[3] = e.z;
                c[4] = kShard ? i + sp.first_instance : i;
            }
            return;
        }
#pragma unroll
        for (int j = J0; j < J1; j++) {
            if (!((vis_bits >> j) & 1u)) continue;
            const uint32_t i = b + (uint32_t)(j * THREADS + t);
            const uint32_t r = (rf == rl) ? rf : region_of(offsets, rf, rl + 1, i);
            const uint32_t start = (r == rf) ? start_f : offsets[r];
            const uint32_t ei = excl(sm, i - b);
            const uint32_t slot = (start >= b) ? start + (ei - excl(sm, start - b)) : start + carry + ei;
            uint32_t out = slot;
            if (kShard) out = (slot < n) ? __ldg(sp.dst_base + r) + (slot - start) : 0xffffffffu;
            if (slot >= n || (kShard && out >= sp.capacity)) {
                atomicOr(error, CADR_DEVERR_BAD_INDEX);
                continue;
            }
            if (!CADR_CHECKED(in_region(offsets, r, i, slot), error)) continue;
            const uint4 e = ent[j - J0];
            uint32_t* c = cmds + (size_t)out * 5;
            c[0] = e.x;
            c[1] = 1u;
            c[2] = e.y;
            c[3] = e.z;
            c[4] = kShard ? i + sp.first_instance : i;
        }
    }

    // Every thread: the counts of the regions ending in this tile (the
    // scan's first tile also writes the zero counts of empty regions).
    __device__ static __forceinline__ void write_counts(const Smem& sm, uint32_t b, uint32_t n, bool first_tile,
                                                        const uint32_t* __restrict__ offsets, uint32_t S,
                                                        uint32_t* __restrict__ counts, uint32_t* error)
    {
        const int t = threadIdx.x;
        const uint32_t carry = sm.info[2], rf = sm.info[4], rl = sm.info[5];
        const uint32_t e_tile = min(b + (uint32_t)SIZE, n);
        for (uint32_t k = rf + (uint32_t)t; k <= rl; k += THREADS) {
            const uint32_t sk = offsets[k], ek = offsets[k + 1];
            if (ek > sk && ek > b && ek <= e_tile) {
                const uint32_t ee = excl(sm, ek - b);
                const uint32_t c = (sk >= b) ? ee - excl(sm, sk - b) : carry + ee;
                if (CADR_CHECKED(c <= ek - sk, error)) counts[k] = c;
            }
        }
        if (first_tile)
            for (uint32_t k = (uint32_t)t; k < S; k += THREADS)
                if (offsets[k] == offsets[k + 1]) counts[k] = 0u;
    }
};

using LeafTile = Tile<kLeafThreads, kLeafIpt>;

// The tile word of a reduce-then-scan pass: the visible drawables of the
// tile's last StateSet region that lie in the tile (all of the tile's
// visible drawables when no region starts in it), and in bit 31 whether a
// region starts in the tile.
constexpr uint32_t kTileHead = 0x80000000u;

// Warp 0 (all lanes return it): the tile word of the tile of drawables
// [b, b + kLeafTile) from its ballots (ballot[j][w] covers the tile's
// drawables [32 (j kLeafWarps + w), + 32)) and the start of the region
// holding its last drawable.
__device__ __forceinline__ uint32_t leaf_tile_word(const uint32_t (*ballot)[kLeafWarps], uint32_t last_start,
                                                   uint32_t b)
{
    const int lane = threadIdx.x & 31;
    const bool head = last_start >= b;
    const uint32_t q = head ? last_start - b : 0u;
    uint32_t total = 0, before = 0;
#pragma unroll
    for (int h = 0; h < (kLeafIpt * kLeafWarps) / kWarp; h++) {
        const uint32_t k = (uint32_t)(lane + h * kWarp);
        const uint32_t v = ballot[k / kLeafWarps][k % kLeafWarps];
        total += __popc(v);
        if (32u * k + 32u <= q)
            before += __popc(v);
        else if (32u * k < q)
            before += __popc(v & ((1u << (q - 32u * k)) - 1u));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        total += __shfl_xor_sync(~0u, total, o);
        before += __shfl_xor_sync(~0u, before, o);
    }
    return head ? (total - before) | kTileHead : total;
}

// One CTA of THREADS threads replaces the tile words [lo, hi) by their
// carries: the visible drawables of the region holding the tile's first
// drawable that precede the tile.  A segmented exclusive scan in chunks of
// THREADS * PER tiles; a region start in a tile restarts the sum at that
// tile's count, and the first tile's carry is 0.  With kVec (words + lo
// 16-byte aligned) a thread's PER words move as 16-byte vectors.
template <int THREADS, int PER, bool kVec = false>
__device__ __forceinline__ void scan_tile_words(uint32_t* __restrict__ words, uint32_t lo, uint32_t hi)
{
    __shared__ uint32_t s_val[THREADS / kWarp], s_head[THREADS / kWarp];
    __shared__ uint32_t s_run;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t == 0) s_run = 0;
    __syncthreads();
    for (uint32_t c0 = lo; c0 < hi; c0 += (uint32_t)(THREADS * PER)) {
        uint32_t w[PER];
        uint32_t v = 0, h = 0;  // this thread's segmented total and whether it holds a head
        const uint32_t i0 = c0 + (uint32_t)(t * PER);
        const bool vec = kVec && (PER % 4 == 0) && i0 + PER <= hi;
        if (vec) {
#pragma unroll
            for (int k = 0; k < PER; k += 4) {
                const uint4 q = *reinterpret_cast<const uint4*>(words + i0 + k);
                w[k] = q.x; w[k + 1] = q.y; w[k + 2] = q.z; w[k + 3] = q.w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < PER; k++) w[k] = i0 + k < hi ? words[i0 + k] : 0u;
        }
#pragma unroll
        for (int k = 0; k < PER; k++) {
            if (w[k] & kTileHead) {
                v = w[k] & ~kTileHead;
                h = 1;
            } else {
                v += w[k];
            }
        }
        // Inclusive warp scan of (head, value) pairs: a later head resets.
        uint32_t iv = v, ih = h;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t pv = __shfl_up_sync(~0u, iv, o), ph = __shfl_up_sync(~0u, ih, o);
            if (lane >= o && !ih) {
                iv += pv;
                ih = ph;
            }
        }
        if (lane == 31) {
            s_val[warp] = iv;
            s_head[warp] = ih;
        }
        __syncthreads();
        if (warp == 0) {
            uint32_t wv = lane < THREADS / kWarp ? s_val[lane] : 0u, wh = lane < THREADS / kWarp ? s_head[lane] : 0u;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t pv = __shfl_up_sync(~0u, wv, o), ph = __shfl_up_sync(~0u, wh, o);
                if (lane >= o && !wh) {
                    wv += pv;
                    wh = ph;
                }
            }
            if (lane < THREADS / kWarp) {
                s_val[lane] = wv;  // inclusive over warps 0..lane
                s_head[lane] = wh;
            }
        }
        __syncthreads();
        // Exclusive prefix of this thread: chunk carry-in, earlier warps, earlier lanes.
        uint32_t ev = s_run;
        if (warp > 0) {
            const uint32_t pv = s_val[warp - 1], ph = s_head[warp - 1];
            ev = ph ? pv : ev + pv;
        }
        {
            const uint32_t pv = __shfl_up_sync(~0u, iv, 1), ph = __shfl_up_sync(~0u, ih, 1);
            if (lane > 0) ev = ph ? pv : ev + pv;
        }
        uint32_t run = ev;
        uint32_t o[PER];
#pragma unroll
        for (int k = 0; k < PER; k++) {
            o[k] = run;
            run = (w[k] & kTileHead) ? (w[k] & ~kTileHead) : run + w[k];
        }
        if (vec) {
#pragma unroll
            for (int k = 0; k < PER; k += 4)
                *reinterpret_cast<uint4*>(words + i0 + k) = make_uint4(o[k], o[k + 1], o[k + 2], o[k + 3]);
        } else {
#pragma unroll
            for (int k = 0; k < PER; k++)
                if (i0 + k < hi) words[i0 + k] = o[k];
        }
        __syncthreads();
        if (t == THREADS - 1) s_run = run;
        __syncthreads();
    }
}

// Called by thread 0 of every CTA as its last action: the last CTA of the
// launch re-arms the control block for the next pass.
__device__ __forceinline__ void finish_pass(LookbackCtl* ctl)
{
    __threadfence();
    const uint32_t old = atomicAdd(&ctl->done_counter, 1u);
    if (old == gridDim.x - 1) {
        atomicExch(&ctl->tile_counter, 0u);
        atomicExch(&ctl->done_counter, 0u);
        atomicAdd(&ctl->epoch, 1u);
    }
}

}  // namespace cadr
