// The persistent step kernel: one launch advances every scene of a batch by one
// pbd_simulate_with_constraints call (src/physics/pbd.cpp:468-747).
//
// Execution groups. A scene is processed by a group of threads that synchronises between the
// phases of the step:
//   CtaGroup   one CTA per scene (batches of small scenes; barrier = __syncthreads)
//   GridGroup  every CTA of a cooperative launch on one large scene (barrier = a bounded
//              grid-wide barrier; the launch is cooperative, so all CTAs are co-resident)
//
// Phases of one step:
//   broad phase   exact pair list in the reference's order (FP32 prefilter, FP64 test with
//                 round-to-nearest intrinsics and no contraction, so it is bit-identical)
//   islands       lock-free union-find and the sleeping update (pbd.cpp:477-506)
//   schedule      order-preserving graph colouring of the Gauss–Seidel sweep: node k (an external
//                 constraint or a broad-phase pair) gets level 1 + max(level of the previous node
//                 on each of its non-fixed bodies). Nodes of one level share no non-fixed body, and
//                 every pair of nodes that does share one keeps the reference's relative order, so
//                 sweeping level by level reproduces the serial sweep (pbd.cpp:615-620) exactly.
//   substeps      predict, hull transform, warp-per-pair narrowphase, level-by-level position
//                 solve, velocity update, level-by-level velocity solve.
#pragma once
#include "rp_math.cuh"
#include "rp_world.h"
#include "rp_narrow.cuh"
#include "rp_solve.cuh"
#include <type_traits>

namespace rp {

constexpr int BLOCK = 256;
constexpr int WARPS_PER_BLOCK = BLOCK / 32;
// ---------------------------------------------------------------------------------------------
// Groups
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// True once a bounded wait of this frame has given up (the status word of scene 0 carries the bit;
// only the cooperative grid, which steps a world of one scene, waits at grid barriers). Every kernel
// of the frame then returns at once, so no kernel works on data a skipped phase never wrote.
__device__ __forceinline__ bool frame_abandoned(const uint32_t* status) {
    return (*(const volatile uint32_t*)status & ST_BARRIER_TIMEOUT) != 0;
}

// Grid barrier of a cooperative launch: one arrival counter that only grows. The host zeroes it
// before every frame (and before every other launch sequence that uses it), and every cooperative
// kernel of a sequence has the same number of CTAs, so after k complete barriers the counter is
// k * gridDim.x: a CTA arriving at count `old` waits until the count reaches the next multiple of
// gridDim.x. One atomic per CTA and nothing else on the release path (no reset, no generation word).
// The wait is bounded by limit_ns of the globaltimer (checked every 64 polls; 0 gives up at the first
// check that finds the barrier incomplete), and it also ends when another CTA has given up. A CTA
// that gives up sets ST_BARRIER_TIMEOUT and leaves the launch (every thread exits together), so it
// never runs a phase on data the others have not finished; the CTAs still waiting for it give up in
// turn, and the frame's later kernels return at once (frame_abandoned).
static __device__ __noinline__ void grid_barrier(unsigned* bar, uint32_t* status, unsigned long long limit_ns) {
    __shared__ int s_gave_up;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned nb = gridDim.x;
        __threadfence();                                   // this CTA's writes before its arrival
        const unsigned old = atomicAdd(&bar[0], 1u);
        const unsigned target = old - old % nb + nb;
        int gave_up = 0;
        if ((int)(ld_acquire_gpu(&bar[0]) - target) < 0) {
            if (limit_ns == 0) gave_up = 1;
            const unsigned long long t0 = global_ns();
            unsigned polls = 0;
            while (!gave_up && (int)(ld_acquire_gpu(&bar[0]) - target) < 0) {
                __nanosleep(32);
                if ((++polls & 63u) == 0u && (global_ns() - t0 > limit_ns || frame_abandoned(status))) gave_up = 1;
            }
        }
        if (gave_up) atomicOr(status, (uint32_t)ST_BARRIER_TIMEOUT);
        __threadfence();
        s_gave_up = gave_up;
    }
    __syncthreads();
    if (s_gave_up) asm volatile("exit;");
}

// Records the first degenerate condition of the world (ST_DEG_* bits, scene, pair, substep) for
// rp_degenerate_info; later ones only set status bits.
template <typename R>
__device__ __forceinline__ void note_degenerate(const WorldView<R>& W, uint32_t bits, int s, int a, int b) {
    const uint32_t deg = bits & (uint32_t)ST_DEG_MASK;
    if (deg == 0u || !W.deg_first) return;
    if (atomicCAS(reinterpret_cast<unsigned*>(W.deg_first), 0u, deg) == 0u) {
        W.deg_first[1] = s;
        W.deg_first[2] = a;
        W.deg_first[3] = b;
        W.deg_first[4] = W.queue ? W.queue[4] : -1;
    }
}

struct CtaGroup {
    __device__ int rank() const { return (int)threadIdx.x; }
    __device__ int size() const { return (int)blockDim.x; }
    __device__ int nblocks() const { return 1; }
    __device__ int block() const { return 0; }
    __device__ void sync() const { __syncthreads(); }
};

struct WarpGroup {   // one warp per scene (small scenes of a batch; barrier = __syncwarp)
    __device__ int rank() const { return (int)(threadIdx.x & 31); }
    __device__ int size() const { return 32; }
    __device__ int nblocks() const { return 1; }
    __device__ int block() const { return 0; }
    __device__ void sync() const { __syncwarp(); }
};

struct GridGroup {
    unsigned* bar;
    uint32_t* status;
    unsigned long long limit_ns;
    __device__ int rank() const { return (int)(blockIdx.x * blockDim.x + threadIdx.x); }
    __device__ int size() const { return (int)(gridDim.x * blockDim.x); }
    __device__ int nblocks() const { return (int)gridDim.x; }
    __device__ int block() const { return (int)blockIdx.x; }
    __device__ void sync() const { grid_barrier(bar, status, limit_ns); }
};

// Block-wide inclusive scan of one value per thread; smem must hold 32 ints.
static __device__ int block_incl_scan(int x, int* smem, int& total) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int v = warp_incl_scan(x);
    if (lane == 31) smem[wid] = v;
    __syncthreads();
    if (wid == 0) {
        int nw = (blockDim.x + 31) >> 5;
        int t = lane < nw ? smem[lane] : 0;
        t = warp_incl_scan(t);
        if (lane < nw) smem[lane] = t;
    }
    __syncthreads();
    int add = wid > 0 ? smem[wid - 1] : 0;
    total = smem[((blockDim.x + 31) >> 5) - 1];
    __syncthreads();
    return v + add;
}

// Group-wide exclusive scan of data[0, n) in place; returns the total to every thread.
// tmp: nblocks ints of global scratch (unused for a CTA group).
template <class G>
__device__ int group_exclusive_scan(const G& g, int* data, int n, int* tmp, int* smem) {
    int nb = g.nblocks(), bi = g.block();
    int chunk = (n + nb - 1) / nb;
    int lo = min(n, bi * chunk), hi = min(n, lo + chunk);
    int carry = 0;
    for (int base = lo; base < hi; base += blockDim.x) {
        int i = base + (int)threadIdx.x;
        int x = i < hi ? data[i] : 0;
        int tot;
        int incl = block_incl_scan(x, smem, tot);
        if (i < hi) data[i] = carry + incl - x;
        carry += tot;
    }
    if (nb == 1) {
        __syncthreads();
        return carry;
    }
    if (threadIdx.x == 0) tmp[bi] = carry;
    g.sync();
    int off = 0, total = 0;
    for (int k = (int)(threadIdx.x & 31); k < nb; k += 32) {
        int t = tmp[k];
        total += t;
        if (k < bi) off += t;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        off += __shfl_xor_sync(0xffffffffu, off, o);
        total += __shfl_xor_sync(0xffffffffu, total, o);
    }
    for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) data[i] += off;
    g.sync();
    return total;
}

// ---------------------------------------------------------------------------------------------
// Broad phase (broad.cpp:6-28): all i < j with |p_i - p_j| <= r_i + r_j + 0.1, in row order.
__device__ __forceinline__ bool broad_exact(double4_32a pi, double4_32a pj, double ri, double rj) {
    double dx = __dsub_rn(pi.x, pj.x), dy = __dsub_rn(pi.y, pj.y), dz = __dsub_rn(pi.z, pj.z);
    double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    double dist = __dsqrt_rn(d2);
    double mx = __dadd_rn(__dadd_rn(ri, rj), 0.1);
    return dist <= mx;
}

// Conservative FP32 rejection: true when the pair certainly fails the exact test.
__device__ __forceinline__ bool broad_reject(float4 fi, float4 fj) {
    // fi = (x, y, z, r + 0.05) rounded to float; w absorbs the 0.1 margin split between the two
    float bx = 2.5e-7f * (fabsf(fi.x) + fabsf(fj.x)) + 1e-6f;
    float by = 2.5e-7f * (fabsf(fi.y) + fabsf(fj.y)) + 1e-6f;
    float bz = 2.5e-7f * (fabsf(fi.z) + fabsf(fj.z)) + 1e-6f;
    float dx = fmaxf(fabsf(fi.x - fj.x) - bx, 0.f), dy = fmaxf(fabsf(fi.y - fj.y) - by, 0.f),
          dz = fmaxf(fabsf(fi.z - fj.z) - bz, 0.f);
    float mx = (fi.w + fj.w) * 1.00001f + 1e-6f;
    return dx * dx + dy * dy + dz * dz > mx * mx;
}

// Order-preserving map of a float onto an unsigned key (negative values reversed).
__device__ __forceinline__ uint32_t float_key(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Scenes of this many bodies take the sort-based broad phase when a grid group steps them (the upper
// bound keeps a row's bitmap of second indices within the block's shared scratch).
constexpr int SORTED_BROAD_MIN = 1024;
constexpr int SORTED_BROAD_MAX = 65536;
// Up to this many bodies one CTA does the radix sort alone.
constexpr int SORT_ONE_CTA_MAX = 16384;

// Sort-based broad phase of one large scene on a grid group (broad.cpp:6-28). Every body gets the x
// interval [x - r - 0.05, x + r + 0.05], rounded outwards to float; two bodies can pass the exact test
// |p_i - p_j| <= r_i + r_j + 0.1 only if their intervals overlap. The bodies are sorted by the lower
// end of their interval (LSD radix sort, four 8-bit digits, each pass a per-tile histogram, a group
// scan and a stable tile scatter), then one warp per sorted body scans the bodies that follow it while
// their interval starts before its interval ends, and applies the exact test (FP32 rejection first,
// then the reference's FP64 arithmetic). Hits are counted per row (the lower body index), the counts
// scanned into row offsets, the hits placed, and each row sorted by its second index: the pair list
// and its order are the reference's.
template <typename R>
__device__ void broad_phase_sorted(const WorldView<R>& W, const GridGroup& g, int s, int* smem) {
    __shared__ int s_cnt[WARPS_PER_BLOCK][256];
    const int b0 = W.scene_body[s], n = W.scene_body[s + 1] - b0;
    const int ntot = W.scene_body[W.num_scenes];
    const int pcap = W.scene_pair_cap[s + 1] - W.scene_pair_cap[s];
    int2* pairs = W.pairs + W.scene_pair_cap[s];
    const int tiles = (n + BLOCK - 1) / BLOCK;
    uint32_t* key[2] = {W.sort_key + b0, W.sort_key + ntot + b0};
    int* val[2] = {W.sort_val + b0, W.sort_val + ntot + b0};
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int i = g.rank(); i < n; i += g.size()) {
        const double4_32a p = W.pos[b0 + i];
        const double r = W.radius[b0 + i];
        const double slack = 1e-6 * (1.0 + fabs(p.x) + r);
        key[0][i] = float_key(__double2float_rd(p.x - r - 0.05 - slack));
        val[0][i] = i;
        W.sort_hi[b0 + i] = __double2float_ru(p.x + r + 0.05 + slack);
        W.row_count[b0 + i] = 0;
        W.body_tl_count[b0 + i] = 0;
    }
    g.sync();
    if (n <= SORT_ONE_CTA_MAX) {
        // one CTA sorts (the radix passes then need block barriers only); the others wait once
        if (g.block() == 0) {
            __shared__ int s_base[256];
            int cur = 0;
            for (int shift = 0; shift < 32; shift += 8) {
                s_base[threadIdx.x] = 0;
                __syncthreads();
                for (int i = threadIdx.x; i < n; i += blockDim.x) atomicAdd(&s_base[(key[cur][i] >> shift) & 255u], 1);
                __syncthreads();
                int tot;
                const int x = s_base[threadIdx.x];
                const int incl = block_incl_scan(x, smem, tot);
                s_base[threadIdx.x] = incl - x;
                __syncthreads();
                for (int t = 0; t < tiles; ++t) {
                    for (int d = lane; d < 256; d += 32) s_cnt[wid][d] = 0;
                    __syncthreads();
                    const int i = t * BLOCK + (int)threadIdx.x;
                    uint32_t k = 0;
                    int v = 0, d = -1;
                    if (i < n) { k = key[cur][i]; v = val[cur][i]; d = (int)((k >> shift) & 255u); }
                    const unsigned peers = __match_any_sync(0xffffffffu, d);
                    const int rank = __popc(peers & ((1u << lane) - 1u));
                    if (d >= 0 && rank == 0) s_cnt[wid][d] = __popc(peers);
                    __syncthreads();
                    if (d >= 0) {
                        int before = 0;
                        for (int w2 = 0; w2 < wid; ++w2) before += s_cnt[w2][d];
                        const int pos = s_base[d] + before + rank;
                        key[cur ^ 1][pos] = k;
                        val[cur ^ 1][pos] = v;
                    }
                    __syncthreads();
                    int add = 0;
                    for (int w2 = 0; w2 < WARPS_PER_BLOCK; ++w2) add += s_cnt[w2][threadIdx.x];
                    s_base[threadIdx.x] += add;
                    __syncthreads();
                }
                cur ^= 1;
            }
        }
        g.sync();
    } else {
        int cur = 0;
        for (int shift = 0; shift < 32; shift += 8) {
            for (int t = g.block(); t < tiles; t += g.nblocks()) {
                for (int d = threadIdx.x; d < 256; d += blockDim.x) s_cnt[0][d] = 0;
                __syncthreads();
                const int i = t * BLOCK + (int)threadIdx.x;
                if (i < n) atomicAdd(&s_cnt[0][(key[cur][i] >> shift) & 255u], 1);
                __syncthreads();
                for (int d = threadIdx.x; d < 256; d += blockDim.x) W.sort_hist[d * tiles + t] = s_cnt[0][d];
                __syncthreads();
            }
            g.sync();
            group_exclusive_scan(g, W.sort_hist, 256 * tiles, W.scan_tmp, smem);
            for (int t = g.block(); t < tiles; t += g.nblocks()) {
                for (int d = lane; d < 256; d += 32) s_cnt[wid][d] = 0;
                __syncthreads();
                const int i = t * BLOCK + (int)threadIdx.x;
                uint32_t k = 0;
                int v = 0, d = -1;
                if (i < n) { k = key[cur][i]; v = val[cur][i]; d = (int)((k >> shift) & 255u); }
                const unsigned peers = __match_any_sync(0xffffffffu, d);
                const int rank = __popc(peers & ((1u << lane) - 1u));
                if (d >= 0 && rank == 0) s_cnt[wid][d] = __popc(peers);
                __syncthreads();
                if (d >= 0) {
                    int before = 0;
                    for (int w2 = 0; w2 < wid; ++w2) before += s_cnt[w2][d];
                    const int pos = W.sort_hist[d * tiles + t] + before + rank;
                    key[cur ^ 1][pos] = k;
                    val[cur ^ 1][pos] = v;
                }
                __syncthreads();
            }
            g.sync();
            cur ^= 1;
        }
    }
    // sweep: count hits per row, scan, then place them
    const int gw = g.rank() >> 5, nw = g.size() >> 5;
    int total = 0;
    for (int pass = 0; pass < 2; ++pass) {
        for (int i = gw; i < n; i += nw) {
            const int a = val[0][i];
            const uint32_t hik = float_key(W.sort_hi[b0 + a]);
            const double4_32a pa = W.pos[b0 + a];
            const double ra = W.radius[b0 + a];
            const float4 fa = make_float4((float)pa.x, (float)pa.y, (float)pa.z, (float)ra + 0.05f);
            for (int kb = i + 1; kb < n; kb += 32) {
                const int k = kb + lane;
                const bool in = k < n && key[0][k] <= hik;
                if (in) {
                    const int b = val[0][k];
                    const double4_32a pb = W.pos[b0 + b];
                    const double rb = W.radius[b0 + b];
                    const float4 fb = make_float4((float)pb.x, (float)pb.y, (float)pb.z, (float)rb + 0.05f);
                    if (!broad_reject(fa, fb) && broad_exact(pa, pb, ra, rb)) {
                        const int lo = min(a, b), hi = max(a, b);
                        if (pass == 0) {
                            atomicAdd(&W.row_count[b0 + lo], 1);
                        } else {
                            const int pos = W.row_count[b0 + lo] + atomicAdd(&W.body_tl_count[b0 + lo], 1);
                            if (pos < pcap) pairs[pos] = make_int2(b0 + lo, b0 + hi);
                        }
                    }
                }
                if (!__any_sync(0xffffffffu, in)) break;
            }
        }
        g.sync();
        if (pass == 0) total = group_exclusive_scan(g, W.row_count + b0, n, W.scan_tmp, smem);
    }
    // each row in increasing second index: short rows by insertion sort, one thread each; long rows
    // (a fixed floor or wall meets nearly every body) by one block each, through a bitmap of the row's
    // second indices whose set bits are then written out in order
    for (int a = g.rank(); a < n; a += g.size()) {
        const int st = W.row_count[b0 + a], cnt = W.body_tl_count[b0 + a];
        if (cnt > 32) continue;
        const int en = min(st + cnt, pcap);
        for (int x = st + 1; x < en; ++x) {
            const int2 v = pairs[x];
            int y = x - 1;
            while (y >= st && pairs[y].y > v.y) { pairs[y + 1] = pairs[y]; --y; }
            pairs[y + 1] = v;
        }
    }
    uint32_t* bits = reinterpret_cast<uint32_t*>(&s_cnt[0][0]);   // n <= 65536: at most 2048 words
    const int nwords = (n + 31) >> 5;
    for (int a = g.block(); a < n; a += g.nblocks()) {
        const int st = W.row_count[b0 + a], cnt = W.body_tl_count[b0 + a];
        if (cnt <= 32) continue;
        for (int k = threadIdx.x; k < nwords; k += blockDim.x) bits[k] = 0u;
        __syncthreads();
        const int en = min(st + cnt, pcap);
        for (int e = st + (int)threadIdx.x; e < en; e += blockDim.x) {
            const int v = pairs[e].y - b0;
            atomicOr(&bits[v >> 5], 1u << (v & 31));
        }
        __syncthreads();
        const int per = (nwords + (int)blockDim.x - 1) / (int)blockDim.x;
        const int w0 = min(nwords, (int)threadIdx.x * per), w1 = min(nwords, w0 + per);
        int mine = 0;
        for (int k = w0; k < w1; ++k) mine += __popc(bits[k]);
        int tot;
        int pos = st + block_incl_scan(mine, smem, tot) - mine;
        for (int k = w0; k < w1; ++k) {
            uint32_t m = bits[k];
            while (m) {
                const int bit = __ffs(m) - 1;
                m &= m - 1u;
                if (pos < pcap) pairs[pos] = make_int2(b0 + a, b0 + (k << 5) + bit);
                ++pos;
            }
        }
        __syncthreads();
    }
    if (g.rank() == 0) {
        W.pair_count[s] = total;
        atomicAdd(&W.counters[5], (unsigned long long)total);
        if (total > pcap) atomicOr(&W.status[s], (uint32_t)ST_PAIR_OVERFLOW);
    }
    g.sync();
}

template <typename R, class G>
__device__ void broad_phase(const WorldView<R>& W, const G& g, int s, int* smem) {
    const int b0 = W.scene_body[s], n = W.scene_body[s + 1] - b0;
    if constexpr (std::is_same<G, GridGroup>::value) {
        if (n >= SORTED_BROAD_MIN && n <= SORTED_BROAD_MAX) { broad_phase_sorted(W, g, s, smem); return; }
    }
    // A CTA stages the scene's FP32 bounds (position, radius + 0.05) in shared memory once, so the
    // FP32 rejection of each of the n(n-1)/2 pairs reads them instead of converting two FP64 poses
    // (FP64 conversions issue at a small fraction of the FP32 rate on GB300); only pairs the
    // rejection keeps load the FP64 poses for the exact test. Same tests, same pairs, same order.
    constexpr int BROAD_STAGE = 1024;
    float4* sf = nullptr;
    if constexpr (std::is_same<G, CtaGroup>::value) {
        __shared__ float4 s_bounds[BROAD_STAGE];
        if (n <= BROAD_STAGE) {
            for (int i = g.rank(); i < n; i += g.size()) {
                const double4_32a p = W.pos[b0 + i];
                s_bounds[i] = make_float4((float)p.x, (float)p.y, (float)p.z, (float)W.radius[b0 + i] + 0.05f);
            }
            sf = s_bounds;
            g.sync();
        }
    }
    auto bound = [&](int i) {
        if (sf) return sf[i];
        const double4_32a p = W.pos[b0 + i];
        return make_float4((float)p.x, (float)p.y, (float)p.z, (float)W.radius[b0 + i] + 0.05f);
    };
    const int pcap = W.scene_pair_cap[s + 1] - W.scene_pair_cap[s];
    int2* pairs = W.pairs + W.scene_pair_cap[s];
    const int lane = threadIdx.x & 31;
    const int gw = g.rank() >> 5, nw = g.size() >> 5;
    // per-row counts (warp per row)
    for (int i = gw; i < n; i += nw) {
        const float4 fi = bound(i);
        int cnt = 0;
        for (int jb = i + 1; jb < n; jb += 32) {
            int j = jb + lane;
            bool hit = false;
            if (j < n && !broad_reject(fi, bound(j)))
                hit = broad_exact(W.pos[b0 + i], W.pos[b0 + j], W.radius[b0 + i], W.radius[b0 + j]);
            cnt += __popc(__ballot_sync(0xffffffffu, hit));
        }
        if (lane == 0) W.row_count[b0 + i] = cnt;
    }
    g.sync();
    int total = group_exclusive_scan(g, W.row_count + b0, n, W.scan_tmp, smem);
    if (g.rank() == 0) {
        W.pair_count[s] = total;
        atomicAdd(&W.counters[5], (unsigned long long)total);
    }
    if (total > pcap) {
        if (g.rank() == 0) atomicOr(&W.status[s], (uint32_t)ST_PAIR_OVERFLOW);
    }
    for (int i = gw; i < n; i += nw) {
        const float4 fi = bound(i);
        int out = W.row_count[b0 + i];
        for (int jb = i + 1; jb < n; jb += 32) {
            int j = jb + lane;
            bool hit = false;
            if (j < n && !broad_reject(fi, bound(j)))
                hit = broad_exact(W.pos[b0 + i], W.pos[b0 + j], W.radius[b0 + i], W.radius[b0 + j]);
            unsigned m = __ballot_sync(0xffffffffu, hit);
            int pos = out + __popc(m & ((1u << lane) - 1u));
            if (hit && pos < pcap) pairs[pos] = make_int2(b0 + i, b0 + j);
            out += __popc(m);
        }
    }
    g.sync();
}

// ---------------------------------------------------------------------------------------------
// Islands and sleeping (broad.cpp:31-116, pbd.cpp:477-506)
__device__ __forceinline__ int uf_find(int* parent_, int x) {
    volatile int* parent = parent_;
    int p = parent[x];
    while (p != x) {
        int gp = parent[p];
        x = p;
        p = gp;
    }
    return x;
}
__device__ __forceinline__ void uf_union(int* parent, int a, int b) {
    for (int guard = 0; guard < (1 << 20); ++guard) {
        int ra = uf_find(parent, a), rb = uf_find(parent, b);
        if (ra == rb) return;
        if (ra < rb) { int t = ra; ra = rb; rb = t; }
        if (atomicCAS(&parent[ra], ra, rb) == ra) return;
    }
}

template <typename R, class G>
__device__ void islands(const WorldView<R>& W, const G& g, int s, double dt) {
    const int b0 = W.scene_body[s], b1 = W.scene_body[s + 1];
    const int np = min(W.pair_count[s], W.scene_pair_cap[s + 1] - W.scene_pair_cap[s]);
    const int2* pairs = W.pairs + W.scene_pair_cap[s];
    const int e0 = W.scene_ext[s], e1 = W.scene_ext[s + 1];
    for (int b = b0 + g.rank(); b < b1; b += g.size()) { W.uf_parent[b] = b; W.island_awake[b] = 0; }
    g.sync();
    for (int k = g.rank(); k < np + (e1 - e0); k += g.size()) {
        int a, c;
        if (k < np) { a = pairs[k].x; c = pairs[k].y; }
        else { a = W.ext[e0 + k - np].e1; c = W.ext[e0 + k - np].e2; }
        if (!W.fixed[a] && !W.fixed[c]) uf_union(W.uf_parent, a, c);
    }
    g.sync();
    for (int b = b0 + g.rank(); b < b1; b += g.size()) {
        if (W.fixed[b]) continue;
        V3<R> v = v3<R>(W.vel[3 * b], W.vel[3 * b + 1], W.vel[3 * b + 2]);
        V3<R> w = v3<R>(W.omega[3 * b], W.omega[3 * b + 1], W.omega[3 * b + 2]);
        R lv = vlen(v), av = vlen(w);
        double d = W.deact[b];
        if (lv < (R)0.10 && av < (R)0.10) d += dt;
        else d = 0.0;
        W.deact[b] = d;
        if (d < 1.0) W.island_awake[uf_find(W.uf_parent, b)] = 1;
    }
    g.sync();
    for (int b = b0 + g.rank(); b < b1; b += g.size()) {
        if (W.fixed[b]) continue;
        W.active[b] = W.island_awake[uf_find(W.uf_parent, b)];
    }
    g.sync();
}

// ---------------------------------------------------------------------------------------------
// The frame's solver nodes (external constraints, then broad-phase pairs, in the reference's
// constraint order): each node's dynamic bodies, and every dynamic body's timeline (the nodes that
// touch it, in constraint order). The per-substep schedules below are built from these.
template <typename R, class G>
__device__ void schedule(const WorldView<R>& W, const G& g, int s, int* smem) {
    const int b0 = W.scene_body[s], nb = W.scene_body[s + 1] - b0;
    const int np = min(W.pair_count[s], W.scene_pair_cap[s + 1] - W.scene_pair_cap[s]);
    const int2* pairs = W.pairs + W.scene_pair_cap[s];
    const int e0 = W.scene_ext[s], ne = W.scene_ext[s + 1] - e0;
    const int nbase = W.scene_node_cap[s];
    const int nn = ne + np;
    int* nbody = W.node_body + 2 * nbase;
    int* tl = W.body_tl + 2 * nbase;
    for (int b = g.rank(); b < nb; b += g.size()) W.body_tl_count[b0 + b] = 0;
    if (g.rank() == 0) W.scene_nodes[s] = nn;
    g.sync();
    for (int k = g.rank(); k < nn; k += g.size()) {
        int a, c;
        bool live = true;
        if (k < ne) { a = W.ext[e0 + k].e1; c = W.ext[e0 + k].e2; }
        else {
            a = pairs[k - ne].x; c = pairs[k - ne].y;
            live = !((W.fixed[a] || !W.active[a]) && (W.fixed[c] || !W.active[c]));
        }
        int ba = (live && !W.fixed[a]) ? a : -1;
        int bc = (live && !W.fixed[c] && c != a) ? c : -1;
        nbody[2 * k] = ba;
        nbody[2 * k + 1] = bc;
        if (ba >= 0) atomicAdd(&W.body_tl_count[ba], 1);
        if (bc >= 0) atomicAdd(&W.body_tl_count[bc], 1);
    }
    g.sync();
    // timeline starts (relative to the scene's timeline base) live in body_tl_start
    for (int b = g.rank(); b < nb; b += g.size()) W.body_tl_start[b0 + b] = W.body_tl_count[b0 + b];
    g.sync();
    group_exclusive_scan(g, W.body_tl_start + b0, nb, W.scan_tmp, smem);
    for (int b = g.rank(); b < nb; b += g.size()) W.body_tl_count[b0 + b] = 0;
    g.sync();
    for (int k = g.rank(); k < nn; k += g.size()) {
        for (int side = 0; side < 2; ++side) {
            int b = nbody[2 * k + side];
            if (b < 0) continue;
            int slot = atomicAdd(&W.body_tl_count[b], 1);
            tl[W.body_tl_start[b] + slot] = k;
        }
    }
    g.sync();
    // sort every timeline (short: a body's broad-phase degree) into constraint order
    for (int b = g.rank(); b < nb; b += g.size()) {
        int st = W.body_tl_start[b0 + b], cnt = W.body_tl_count[b0 + b];
        int* t = tl + st;
        for (int i = 1; i < cnt; ++i) {
            int key = t[i], j = i - 1;
            while (j >= 0 && t[j] > key) { t[j + 1] = t[j]; --j; }
            t[j + 1] = key;
        }
    }
    g.sync();
}

// ---------------------------------------------------------------------------------------------
// Per-substep schedules of the two Gauss–Seidel sweeps, built after the substep's narrowphase.
//
// A node is active in the position sweep (schedule 0) when it is an external constraint or a pair
// with contacts this substep, and in the velocity sweep (schedule 1) when it is a pair with contacts;
// every other node is a no-op there (solve_node / vsolve_node return at once). An active node's
// predecessor on each of its dynamic bodies is the previous active node of that body's timeline.
//
// Reference order (SWEEP_REFERENCE): a node's level is the longest path to it over those links.
// Nodes of one level share no dynamic body, and nodes that share one keep their constraint order,
// so sweeping level by level reproduces the reference's serial sweep (pbd.cpp:615-620, 646-740)
// exactly; leaving the no-op nodes out of the chains only removes waits that did nothing.
//
// Coloured order (SWEEP_COLOURED): a proper colouring of the active nodes (nodes sharing a dynamic
// body get different colours) by Jones–Plassmann rounds with hashed priorities: an uncoloured node
// whose uncoloured neighbours all have lower priority takes the smallest colour its neighbours do
// not use. Sweeping colour by colour is a Gauss–Seidel sweep in another order (not the reference's),
// with far fewer dependent steps: a joint chain takes two or three colours instead of one level per
// link.
enum { SWEEP_REFERENCE = 0, SWEEP_COLOURED = 1 };
constexpr int COLOUR_WORDS = 2;                  // colours 0..127 from the mask; beyond, 128 + round
constexpr int RESCHED_ONE_CTA = 8192;            // grid group: at most this many active nodes relax on one CTA

__device__ __forceinline__ uint32_t node_priority(int k, int salt) {
    uint32_t x = (uint32_t)k * 0x9E3779B1u + (uint32_t)salt * 0x85EBCA77u;
    x ^= x >> 15;
    x *= 0x2C1B3C6Du;
    x ^= x >> 12;
    return x;
}

// "Does any thread of the relaxing sub-group see a change?" and a barrier of that sub-group.
struct SubWarp {
    __device__ int rank() const { return (int)(threadIdx.x & 31); }
    __device__ int size() const { return 32; }
    __device__ bool any(bool c, int*) const {
        __syncwarp();   // orders the lanes' writes of this round before the next round's reads
        return __any_sync(0xffffffffu, c) != 0;
    }
    __device__ void sync() const { __syncwarp(); }
};
struct SubBlock {
    __device__ int rank() const { return (int)threadIdx.x; }
    __device__ int size() const { return (int)blockDim.x; }
    __device__ bool any(bool c, int*) const { return __syncthreads_or(c) != 0; }
    __device__ void sync() const { __syncthreads(); }
};
struct SubGrid {   // the whole cooperative grid; `flags`: three words of global scratch, zeroed
    GridGroup g;
    mutable int round = 0;
    __device__ int rank() const { return g.rank(); }
    __device__ int size() const { return g.size(); }
    __device__ bool any(bool c, int* flags) const {
        // three rotating flags: the one cleared in round r was last read in round r - 2
        if (g.rank() == 0) flags[(round + 1) % 3] = 0;
        if (c) flags[round % 3] = 1;
        g.sync();
        const bool r = ((volatile int*)flags)[round % 3] != 0;
        ++round;
        return r;
    }
    __device__ void sync() const { g.sync(); }
};

template <typename R>
struct SchedView {   // one of the two schedules of scene s
    int* pred;       // [2 * nodes] (scene base applied)
    int* lev;        // [nodes]
    int* count;      // [max_levels + 1]
    int* fill;       // [max_levels + 1]; the last three words are relaxation flags
    int* nodes;      // [nodes] (scene base applied)
    int* list;       // [nodes] active nodes, unordered
    int* levels;     // number of levels of the scene
    int* active;     // number of active nodes of the scene
};

template <typename R>
__device__ __forceinline__ SchedView<R> sched_view(const WorldView<R>& W, int s, int which) {
    const int nbase = W.scene_node_cap[s];
    SchedView<R> v;
    v.pred = (which ? W.node_vpred : W.node_pred) + 2 * nbase;
    v.lev = (which ? W.node_vlevel : W.node_level) + nbase;
    v.count = (which ? W.vlevel_count : W.level_count) + s * (W.max_levels + 1);
    v.fill = (which ? W.vlevel_fill : W.level_fill) + s * (W.max_levels + 1);
    v.nodes = (which ? W.vlevel_nodes : W.level_nodes) + nbase;
    v.list = W.act_list + (size_t)which * W.scene_node_cap[W.num_scenes] + nbase;
    v.levels = (which ? W.scene_vlevels : W.scene_levels) + s;
    v.active = W.act_count + 2 * s + which;
    return v;
}

// Levels (reference order) or colours (coloured order) of one schedule's active nodes, by sub-group q.
template <typename R, class Q>
__device__ void relax_schedule(const WorldView<R>& W, const Q& q, int s, const SchedView<R>& v, int n, int order) {
    const int nbase = W.scene_node_cap[s];
    const int* nbody = W.node_body + 2 * nbase;
    const int* tl = W.body_tl + 2 * nbase;
    volatile int* lev = v.lev;
    int* flags = v.fill + W.max_levels - 2;
    if (order == SWEEP_REFERENCE) {
        for (int round = 0;; ++round) {
            bool changed = false;
            for (int i = q.rank(); i < n; i += q.size()) {
                const int k = v.list[i];
                const int p0 = v.pred[2 * k], p1 = v.pred[2 * k + 1];
                const int l0 = p0 >= 0 ? lev[p0] : -1, l1 = p1 >= 0 ? lev[p1] : -1;
                const int nl = max(l0, l1) + 1;
                if (nl > lev[k]) { lev[k] = nl; changed = true; }
            }
            if (!q.any(changed, flags)) break;
            if (round >= W.max_levels) {
                if (q.rank() == 0) atomicOr(&W.status[s], (uint32_t)ST_LEVEL_OVERFLOW);
                break;
            }
        }
        return;
    }
    // coloured: lev = -2 while uncoloured
    for (int round = 0;; ++round) {
        bool pending = false;
        for (int i = q.rank(); i < n; i += q.size()) {
            const int k = v.list[i];
            if (lev[k] != -2) continue;
            const uint32_t pk = node_priority(k, s);
            uint32_t used[COLOUR_WORDS] = {0u, 0u};
            bool ready = true;
            for (int side = 0; side < 2 && ready; ++side) {
                const int b = nbody[2 * k + side];
                if (b < 0) continue;
                const int st = W.body_tl_start[b], cnt = W.body_tl_count[b];
                for (int t = 0; t < cnt; ++t) {
                    const int j = tl[st + t];
                    if (j == k) continue;
                    const int lj = lev[j];
                    if (lj == -1) continue;                       // not active in this schedule
                    if (lj == -2) {
                        const uint32_t pj = node_priority(j, s);
                        if (pj > pk || (pj == pk && j > k)) { ready = false; break; }
                    } else if (lj < 32 * COLOUR_WORDS) {
                        used[lj >> 5] |= 1u << (lj & 31);
                    }
                }
            }
            if (!ready) { pending = true; continue; }
            int c = -1;
            for (int wd = 0; wd < COLOUR_WORDS && c < 0; ++wd)
                if (~used[wd]) c = 32 * wd + __ffs(~used[wd]) - 1;
            if (c < 0) c = 32 * COLOUR_WORDS + round;             // every small colour taken
            lev[k] = c;
        }
        if (!q.any(pending, flags)) break;
        if (round >= W.max_levels - 32 * COLOUR_WORDS - 4) {
            if (q.rank() == 0) atomicOr(&W.status[s], (uint32_t)ST_LEVEL_OVERFLOW);
            break;
        }
    }
}

// Buckets one schedule's active nodes by level / colour into v.nodes, by sub-group q.
template <typename R, class Q>
__device__ void bucket_schedule(const WorldView<R>& W, const Q& q, int s, const SchedView<R>& v, int n, bool count_levels) {
    int maxl = -1;
    for (int i = q.rank(); i < n; i += q.size()) {
        const int l = v.lev[v.list[i]];
        if (l < 0 || l >= W.max_levels - 3) { atomicOr(&W.status[s], (uint32_t)ST_LEVEL_OVERFLOW); continue; }
        atomicAdd(&v.count[l], 1);
        maxl = max(maxl, l);
    }
    if (maxl >= 0) atomicMax(v.levels, maxl + 1);
    q.sync();
    if (q.rank() == 0) {
        const int L = *v.levels;
        if (count_levels) atomicAdd(&W.counters[6], (unsigned long long)L);
        int acc = 0;
        for (int l = 0; l <= L; ++l) { const int c = v.count[l]; v.count[l] = acc; acc += c; }
    }
    q.sync();
    for (int i = q.rank(); i < n; i += q.size()) {
        const int k = v.list[i];
        const int l = v.lev[k];
        if (l < 0 || l >= W.max_levels - 3) continue;
        v.nodes[v.count[l] + atomicAdd(&v.fill[l], 1)] = k;
    }
    q.sync();
}

// Both per-substep schedules of scene s by group g (run after the substep's narrowphase, before the
// position sweep; the per-scene active counters were zeroed by the substep's predict phase).
template <typename R, class G>
__device__ void resched(const WorldView<R>& W, const G& g, int s) {
    const int b0 = W.scene_body[s], nb = W.scene_body[s + 1] - b0;
    const int ne = W.scene_ext[s + 1] - W.scene_ext[s];
    const int nbase = W.scene_node_cap[s];
    const int pbase = W.scene_pair_cap[s];
    const int nn = W.scene_nodes[s];
    const int* nbody = W.node_body + 2 * nbase;
    const int* tl = W.body_tl + 2 * nbase;
    const int order = W.sweep_order;
    const int unset = order == SWEEP_COLOURED ? -2 : 0;
    const SchedView<R> v0 = sched_view(W, s, 0), v1 = sched_view(W, s, 1);
    // the level tables are zero beyond the previous substep's levels (zeroed when the world is built)
    const int used0 = min(*(volatile int*)v0.levels + 1, W.max_levels), used1 = min(*(volatile int*)v1.levels + 1, W.max_levels);
    for (int l = g.rank(); l <= used0; l += g.size()) { v0.count[l] = 0; v0.fill[l] = 0; }
    for (int l = g.rank(); l <= used1; l += g.size()) { v1.count[l] = 0; v1.fill[l] = 0; }
    // predecessor links along every dynamic body's timeline
    for (int b = g.rank(); b < nb; b += g.size()) {
        const int st = W.body_tl_start[b0 + b], cnt = W.body_tl_count[b0 + b];
        int prev0 = -1, prev1 = -1;
        for (int i = 0; i < cnt; ++i) {
            const int k = tl[st + i];
            const int side = nbody[2 * k] == b0 + b ? 0 : 1;
            const bool contacts = k >= ne && W.pair_ccount[pbase + k - ne] > 0;
            if (k < ne || contacts) { v0.pred[2 * k + side] = prev0; prev0 = k; }
            if (contacts) { v1.pred[2 * k + side] = prev1; prev1 = k; }
        }
    }
    // activity per node, the sides without a dynamic body, and the two active lists
    for (int k = g.rank(); k < nn; k += g.size()) {
        const bool live = nbody[2 * k] >= 0 || nbody[2 * k + 1] >= 0;
        const bool contacts = live && k >= ne && W.pair_ccount[pbase + k - ne] > 0;
        const bool a0 = live && (k < ne || contacts);
        v0.lev[k] = a0 ? unset : -1;
        v1.lev[k] = contacts ? unset : -1;
        for (int side = 0; side < 2; ++side)
            if (nbody[2 * k + side] < 0) { v0.pred[2 * k + side] = -1; v1.pred[2 * k + side] = -1; }
        if (a0) v0.list[atomicAdd(v0.active, 1)] = k;
        if (contacts) v1.list[atomicAdd(v1.active, 1)] = k;
    }
    g.sync();
    const int n0 = *(volatile int*)v0.active, n1 = *(volatile int*)v1.active;
    if (g.rank() == 0) { *v0.levels = 0; *v1.levels = 0; }
    if constexpr (std::is_same<G, GridGroup>::value) {
        if (n0 + n1 <= RESCHED_ONE_CTA) {
            if (g.block() == 0) {
                SubBlock q;
                if (n0 + n1 > 0) {
                    relax_schedule(W, q, s, v0, n0, order);
                    relax_schedule(W, q, s, v1, n1, order);
                }
                bucket_schedule(W, q, s, v0, n0, true);
                bucket_schedule(W, q, s, v1, n1, false);
            }
        } else {
            SubGrid q{g};
            if (g.rank() == 0) {
                int* f0 = v0.fill + W.max_levels - 2;
                int* f1 = v1.fill + W.max_levels - 2;
                f0[0] = f0[1] = f0[2] = 0;
                f1[0] = f1[1] = f1[2] = 0;
            }
            g.sync();
            relax_schedule(W, q, s, v0, n0, order);
            relax_schedule(W, q, s, v1, n1, order);
            bucket_schedule(W, q, s, v0, n0, true);
            bucket_schedule(W, q, s, v1, n1, false);
        }
        g.sync();
    } else if constexpr (std::is_same<G, WarpGroup>::value) {
        SubWarp q;
        relax_schedule(W, q, s, v0, n0, order);
        relax_schedule(W, q, s, v1, n1, order);
        bucket_schedule(W, q, s, v0, n0, true);
        bucket_schedule(W, q, s, v1, n1, false);
    } else {
        SubBlock q;
        relax_schedule(W, q, s, v0, n0, order);
        relax_schedule(W, q, s, v1, n1, order);
        bucket_schedule(W, q, s, v0, n0, true);
        bucket_schedule(W, q, s, v1, n1, false);
    }
}

// ---------------------------------------------------------------------------------------------
// Hull transform (colliders_update, collider.cpp:409-446): one collider of body b by `nsub` threads
// (index `lane` among them)
// POSE_F: take the FP32 build's orientation from the predict phase's FP32 copy (pose_f, the same
// rounding of the FP64 quaternion) instead of converting it again in every lane.
template <typename R, bool EXACT, bool POSE_F = false>
__device__ void transform_collider(const WorldView<R>& W, const Collider& col, int b, int lane, int nsub = 32) {
    const Shape sh = W.shapes[col.shape];
    V3<R>* tv = (V3<R>*)(W.tverts) + col.tv_off;
    V3<R>* tn = (V3<R>*)(W.tnorms) + col.tn_off;
    if (EXACT) {
        const double4_32a p4 = W.pos[b], q4 = W.rot[b];
        M4<double> M = model_matrix(qt<double>(q4.x, q4.y, q4.z, q4.w), v3<double>(p4.x, p4.y, p4.z));
        for (int i = lane; i < sh.nv; i += nsub) {
            const double* v = W.shape_verts + 3 * (sh.vert_off + i);
            tv[i] = v3cast<R>(m4_point(M, v3<double>(v[0], v[1], v[2])));
        }
        for (int i = lane; i < sh.nf; i += nsub) {
            const double* nrm = W.face_normal + 3 * (sh.face_off + i);
            tn[i] = v3cast<R>(vnorm(m4_dir(M, v3<double>(nrm[0], nrm[1], nrm[2]))));
        }
    } else {
        Qt<R> q;
        if (POSE_F) {
            const float4 f = W.pose_f[2 * b + 1];
            q = qt<R>(f.x, f.y, f.z, f.w);
        } else {
            const double4_32a q4 = W.rot[b];
            q = qt<R>((R)q4.x, (R)q4.y, (R)q4.z, (R)q4.w);
        }
        M3<R> Rm = qmat3(q);
        for (int i = lane; i < sh.nv; i += nsub) {
            const float* v = W.shape_verts_f + 3 * (sh.vert_off + i);
            tv[i] = mmulv(Rm, v3<R>((R)v[0], (R)v[1], (R)v[2]));
        }
        for (int i = lane; i < sh.nf; i += nsub) {
            const float* nrm = W.face_normal_f + 3 * (sh.face_off + i);
            tn[i] = vnorm(mmulv(Rm, v3<R>((R)nrm[0], (R)nrm[1], (R)nrm[2])));
        }
    }
}

// every collider of scene s
template <typename R, bool EXACT, class G>
__device__ void transform_hulls(const WorldView<R>& W, const G& g, int s, bool include_fixed) {
    const int b0 = W.scene_body[s], b1 = W.scene_body[s + 1];
    const int c0 = W.col_start[b0], c1 = W.col_start[b1];
    const int lane = threadIdx.x & 31;
    const int gw = g.rank() >> 5, nw = g.size() >> 5;
    for (int ci = c0 + gw; ci < c1; ci += nw) {
        const Collider col = W.colliders[ci];
        if (col.type != COL_HULL) continue;
        const int b = W.col_body[ci];
        if (W.fixed[b] && !include_fixed) continue;
        transform_collider<R, EXACT>(W, col, b, lane);
    }
}

// ---------------------------------------------------------------------------------------------
// Narrowphase: one warp per broad-phase pair
template <typename R, bool EXACT>
__device__ ColView<R> make_view(const WorldView<R>& W, int ci, V3<R> center, V3<R> off, const V3<R>* staged, int body) {
    ColView<R> v;
    v.body = body;
    const Collider col = W.colliders[ci];
    v.type = col.type;
    v.radius = (R)col.radius;
    v.center = center;
    v.off = off;
    v.nv = 0;
    v.nf = 0;
    v.shape = nullptr;
    v.verts = nullptr;
    v.norms = nullptr;
    v.staged = false;
    if (col.type == COL_HULL) {
        v.shape = W.shapes + col.shape;
        v.nv = v.shape->nv;
        v.nf = v.shape->nf;
        v.verts = (const V3<R>*)(W.tverts) + col.tv_off;
        v.norms = (const V3<R>*)(W.tnorms) + col.tn_off;
        if (staged && v.nv <= STAGE_V) {
            for (int i = (int)lane_id(); i < v.nv; i += 32) ((V3<R>*)staged)[i] = vadd(v.verts[i], off);
            __syncwarp();
            v.verts = staged;
            v.staged = true;
        }
    }
    return v;
}

// colliders_get_contacts for one body pair (collider.cpp:560-571); contacts land in sm.
template <typename R, bool EXACT>
__device__ void pair_contacts(const WorldView<R>& W, NarrowSmem<R>& sm, int a, int b, bool raw) {
    if (lane_id() == 0) { sm.ncontacts = 0; sm.status = 0; }
    __syncwarp();
    double4_32a pa = W.pos[a], pb = W.pos[b], qa4 = W.rot[a], qb4 = W.rot[b];
    PairFrame<R, EXACT> fr;
    fr.raw = raw;
    V3<R> offa, offb;
    if (EXACT) {
        offa = v3<R>(0, 0, 0);
        offb = v3<R>(0, 0, 0);
        fr.x1 = v3<R>((R)pa.x, (R)pa.y, (R)pa.z);
        fr.x2 = v3<R>((R)pb.x, (R)pb.y, (R)pb.z);
    } else {
        offa = v3<R>(0, 0, 0);
        offb = v3<R>((R)(pb.x - pa.x), (R)(pb.y - pa.y), (R)(pb.z - pa.z));
        fr.x1 = offa;
        fr.x2 = offb;
    }
    fr.q1inv = qinverse(qt<R>((R)qa4.x, (R)qa4.y, (R)qa4.z, (R)qa4.w));
    fr.q2inv = qinverse(qt<R>((R)qb4.x, (R)qb4.y, (R)qb4.z, (R)qb4.w));
    const int ca0 = W.col_start[a], ca1 = W.col_start[a + 1], cb0 = W.col_start[b], cb1 = W.col_start[b + 1];
    for (int ca = ca0; ca < ca1; ++ca) {
        // exact build: stored vertices are world coordinates, sphere centres the body positions;
        // FP32 build: stored vertices are rotated about the body origin, the frame origin is body a
        ColView<R> va = make_view<R, EXACT>(W, ca, EXACT ? fr.x1 : offa, offa, sm.va, a);
        for (int cb = cb0; cb < cb1; ++cb) {
            ColView<R> vb = make_view<R, EXACT>(W, cb, EXACT ? fr.x2 : offb, offb, sm.vb, b);
            collider_contacts<R, EXACT>(sm, W, va, vb, fr, W.counters);
            __syncwarp();
        }
    }
}

// Gap between the box bound of one body and the sphere bound of another (metres, FP32; exact up to
// ~1e-6 relative), and the scale its rounding error is relative to. d: sphere centre minus the box
// body's origin; q: the box body's orientation.
__device__ __forceinline__ float box_sphere_gap_f(float4 c, float4 hx, float dx, float dy, float dz, float4 q, float rs,
                                                  float& scale) {
    const float ux = -q.x, uy = -q.y, uz = -q.z, qw = q.w;
    // rotate d by the inverse of the box body's rotation: v = d + w t + u x t, t = 2 u x d
    const float tx = 2.f * (uy * dz - uz * dy), ty = 2.f * (uz * dx - ux * dz), tz = 2.f * (ux * dy - uy * dx);
    const float vx = dx + qw * tx + (uy * tz - uz * ty);
    const float vy = dy + qw * ty + (uz * tx - ux * tz);
    const float vz = dz + qw * tz + (ux * ty - uy * tx);
    const float ex = fmaxf(fabsf(vx - c.x) - hx.x, 0.f), ey = fmaxf(fabsf(vy - c.y) - hx.y, 0.f),
                ez = fmaxf(fabsf(vz - c.z) - hx.z, 0.f);
    scale = fabsf(dx) + fabsf(dy) + fabsf(dz) + fabsf(c.x) + fabsf(c.y) + fabsf(c.z) + hx.x + hx.y + hx.z + rs;
    return sqrtf(ex * ex + ey * ey + ez * ez) - rs;
}

__device__ __forceinline__ float box_sphere_gap(float4 c, float4 hx, double4_32a pbox, double4_32a qbox, double4_32a psph,
                                                float rs, float& scale) {
    return box_sphere_gap_f(c, hx, (float)(psph.x - pbox.x), (float)(psph.y - pbox.y), (float)(psph.z - pbox.z),
                            make_float4((float)qbox.x, (float)qbox.y, (float)qbox.z, (float)qbox.w), rs, scale);
}

// True only when the hulls of bodies a and b are certainly apart by much more than rounding: the
// box bound of one misses the sphere bound of the other. For such a pair gjk_collides
// (gjk.cpp:350-379) cannot find the origin inside the Minkowski difference and returns false, so
// the pair yields no contact; skipping it changes no result. Non-unit rotations are never skipped.
template <typename R>
__device__ __forceinline__ bool bounds_apart(const WorldView<R>& W, int a, int b) {
    const double4_32a pa = W.pos[a], pb = W.pos[b], qa = W.rot[a], qb = W.rot[b];
    const float4 ca = W.bound[2 * a], ha = W.bound[2 * a + 1], cb = W.bound[2 * b], hb = W.bound[2 * b + 1];
    const double na = qa.x * qa.x + qa.y * qa.y + qa.z * qa.z + qa.w * qa.w;
    const double nb = qb.x * qb.x + qb.y * qb.y + qb.z * qb.z + qb.w * qb.w;
    if (fabs(na - 1.0) > 1e-6 || fabs(nb - 1.0) > 1e-6) return false;
    float scale;
    if (ha.w != 0.f) {
        float gap = box_sphere_gap(ca, ha, pa, qa, pb, cb.w, scale);
        if (gap > 1e-5f * scale + 1e-6f) return true;
    }
    if (hb.w != 0.f) {
        float gap = box_sphere_gap(cb, hb, pb, qb, pa, ca.w, scale);
        if (gap > 1e-5f * scale + 1e-6f) return true;
    }
    return false;
}

// bounds_apart on the FP32 pose copies: the position rounding (<= 6e-8 |p| per component) is
// covered by widening the margin with the bodies' distance from the origin.
template <typename R>
__device__ __forceinline__ bool bounds_apart_f(const WorldView<R>& W, int a, int b) {
    const float4 pa = W.pose_f[2 * a], qa = W.pose_f[2 * a + 1], pb = W.pose_f[2 * b], qb = W.pose_f[2 * b + 1];
    const float4 ca = W.bound[2 * a], ha = W.bound[2 * a + 1], cb = W.bound[2 * b], hb = W.bound[2 * b + 1];
    const float na = qa.x * qa.x + qa.y * qa.y + qa.z * qa.z + qa.w * qa.w;
    const float nb = qb.x * qb.x + qb.y * qb.y + qb.z * qb.z + qb.w * qb.w;
    if (fabsf(na - 1.f) > 1e-5f || fabsf(nb - 1.f) > 1e-5f) return false;
    const float far = 4e-7f * (fabsf(pa.x) + fabsf(pa.y) + fabsf(pa.z) + fabsf(pb.x) + fabsf(pb.y) + fabsf(pb.z));
    const float dx = pb.x - pa.x, dy = pb.y - pa.y, dz = pb.z - pa.z;
    float scale;
    if (ha.w != 0.f) {
        float gap = box_sphere_gap_f(ca, ha, dx, dy, dz, qa, cb.w, scale);
        if (gap > 1e-5f * scale + far + 1e-6f) return true;
    }
    if (hb.w != 0.f) {
        float gap = box_sphere_gap_f(cb, hb, -dx, -dy, -dz, qb, ca.w, scale);
        if (gap > 1e-5f * scale + far + 1e-6f) return true;
    }
    return false;
}

// Pairs are handed out one at a time from a per-scene counter (work[s], reset before the substep's
// predict phase); a warp fetches its next pair while it computes the current one.
template <typename R, bool EXACT, class G>
__device__ void narrowphase(const WorldView<R>& W, const G& g, int s, NarrowSmem<R>& sm) {
    const int np = min(W.pair_count[s], W.scene_pair_cap[s + 1] - W.scene_pair_cap[s]);
    const int pbase = W.scene_pair_cap[s];
    const int cbase = W.scene_contact_cap[s];
    const int ccap = W.scene_contact_cap[s + 1] - cbase;
    const int lane = threadIdx.x & 31;
    unsigned long long cyc_sum = 0, cyc_max = 0, n_full = 0, n_apart = 0, n_contacts = 0;
    int p = 0;
    if (lane == 0) p = atomicAdd(&W.work[s], 1);
    p = __shfl_sync(0xffffffffu, p, 0);
    while (p < np) {
        int next = 0;
        if (lane == 0) next = atomicAdd(&W.work[s], 1);
        int2 pr = W.pairs[pbase + p];
        int a = pr.x, b = pr.y;
        bool live = !((W.fixed[a] || !W.active[a]) && (W.fixed[b] || !W.active[b]));
        bool apart = live && bounds_apart(W, a, b);
        if (!live || apart) {
            if (lane == 0) { W.pair_ccount[pbase + p] = 0; W.pair_cstart[pbase + p] = 0; }
            n_apart += apart;
            p = __shfl_sync(0xffffffffu, next, 0);
            continue;
        }
        const long long t0 = clock64();
        pair_contacts<R, EXACT>(W, sm, a, b, false);
        const unsigned long long dt = (unsigned long long)(clock64() - t0);
        cyc_sum += dt;
        cyc_max = max(cyc_max, dt);
        ++n_full;
        int nc = sm.ncontacts;
        int start = 0;
        if (lane == 0) {
            start = atomicAdd(&W.contact_count[s], nc);
            if (start + nc > ccap) {
                atomicOr(&W.status[s], (uint32_t)ST_CONTACT_OVERFLOW);
                nc = 0;
            }
            if (sm.status) {
                atomicOr(&W.status[s], (uint32_t)sm.status);
                note_degenerate(W, (uint32_t)sm.status, s, a, b);
            }
            n_contacts += nc;
            W.pair_cstart[pbase + p] = start;
            W.pair_ccount[pbase + p] = nc;
        }
        start = __shfl_sync(0xffffffffu, start, 0);
        nc = __shfl_sync(0xffffffffu, nc, 0);
        for (int k = lane; k < nc; k += 32) {
            R* c = W.contacts + 12 * (size_t)(cbase + start + k);
            V3<R> r1 = sm.c_r1[k], r2 = sm.c_r2[k], n = sm.c_n[k];
            c[0] = r1.x; c[1] = r1.y; c[2] = r1.z; c[3] = 0;
            c[4] = r2.x; c[5] = r2.y; c[6] = r2.z; c[7] = 0;
            c[8] = n.x; c[9] = n.y; c[10] = n.z; c[11] = 0;
        }
        __syncwarp();
        p = __shfl_sync(0xffffffffu, next, 0);
    }
    if (lane == 0 && (n_full | n_apart)) {
        if (n_contacts) atomicAdd(&W.counters[3], n_contacts);
        atomicMax(&W.counters[8], cyc_max);
        atomicAdd(&W.counters[9], cyc_sum);
        atomicAdd(&W.counters[10], n_full);
        atomicAdd(&W.counters[11], n_apart);
    }
}

// ---------------------------------------------------------------------------------------------
// Level sweeps
template <typename R, bool EXACT>
__device__ void solve_node(const WorldView<R>& W, int s, int k, R h) {
    const int e0 = W.scene_ext[s], ne = W.scene_ext[s + 1] - e0;
    if (k < ne) {
        if constexpr (EXACT) ext_solve<R, EXACT>(W, W.ext[e0 + k], W.ext_lambda + 4 * (size_t)(e0 + k), h);
        else fext_solve(W, W.ext[e0 + k], W.ext_base[e0 + k], reinterpret_cast<float*>(W.ext_lambda + 4 * (size_t)(e0 + k)), h);
        return;
    }
    const int p = W.scene_pair_cap[s] + (k - ne);
    const int nc = W.pair_ccount[p];
    if (nc == 0) return;
    int2 pr = W.pairs[p];
    const R mus = (W.material[4 * pr.x] + W.material[4 * pr.y]) / (R)2.0f;
    R* c = W.contacts + 12 * (size_t)(W.scene_contact_cap[s] + W.pair_cstart[p]);
    if constexpr (EXACT) {
        Body<R> a = load_body(W, pr.x), b = load_body(W, pr.y);
        for (int i = 0; i < nc; ++i) collision_solve<R, EXACT>(W, a, b, c + 12 * i, h, mus);
        store_pose(W, a);
        store_pose(W, b);
    } else {
        FBody a = load_fbody(W, pr.x), b = load_fbody(W, pr.y);
        const float4 bb = W.pair_base[p];
        const V3<float> base_ab = v3<float>(bb.x, bb.y, bb.z);
        for (int i = 0; i < nc; ++i) fcollision_solve(W, a, b, base_ab, c + 12 * i, mus);
        store_fbody(W, a);
        store_fbody(W, b);
    }
}

template <typename R, bool EXACT>
__device__ void vsolve_node(const WorldView<R>& W, int s, int k, R h) {
    const int ne = W.scene_ext[s + 1] - W.scene_ext[s];
    if (k < ne) return;
    const int p = W.scene_pair_cap[s] + (k - ne);
    const int nc = W.pair_ccount[p];
    if (nc == 0) return;
    int2 pr = W.pairs[p];
    const int ia = pr.x, ib = pr.y;
    // anchors rotated by the current orientations (the FP32 build converts each orientation once)
    Qt<R> qa, qb;
    M3<R> Ia, Ib;
    VelBody<R> a, b;
    {
        if constexpr (EXACT) {
            double4_32a q4a = W.rot[ia], q4b = W.rot[ib];
            qa = qcast<R>(qt<double>(q4a.x, q4a.y, q4a.z, q4a.w));
            qb = qcast<R>(qt<double>(q4b.x, q4b.y, q4b.z, q4b.w));
        } else {   // the FP32 copies the fold wrote: the same casts of the FP64 orientations
            const float4 fa = W.pose_f[2 * ia + 1], fb = W.pose_f[2 * ib + 1];
            qa = qt<R>(fa.x, fa.y, fa.z, fa.w);
            qb = qt<R>(fb.x, fb.y, fb.z, fb.w);
        }
        R sa[6], sb[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) { sa[i] = W.inv_inertia[6 * ia + i]; sb[i] = W.inv_inertia[6 * ib + i]; }
        Ia = world_tensor(qa, msym(sa));
        Ib = world_tensor(qb, msym(sb));
        a.invm = W.inv_mass[ia];
        b.invm = W.inv_mass[ib];
        a.fixed = W.fixed[ia] != 0;
        b.fixed = W.fixed[ib] != 0;
    }
    V3<R> va = v3<R>(W.vel[3 * ia], W.vel[3 * ia + 1], W.vel[3 * ia + 2]);
    V3<R> wa = v3<R>(W.omega[3 * ia], W.omega[3 * ia + 1], W.omega[3 * ia + 2]);
    V3<R> vb = v3<R>(W.vel[3 * ib], W.vel[3 * ib + 1], W.vel[3 * ib + 2]);
    V3<R> wb = v3<R>(W.omega[3 * ib], W.omega[3 * ib + 1], W.omega[3 * ib + 2]);
    V3<R> pva = v3<R>(W.prev_vel[3 * ia], W.prev_vel[3 * ia + 1], W.prev_vel[3 * ia + 2]);
    V3<R> pwa = v3<R>(W.prev_omega[3 * ia], W.prev_omega[3 * ia + 1], W.prev_omega[3 * ia + 2]);
    V3<R> pvb = v3<R>(W.prev_vel[3 * ib], W.prev_vel[3 * ib + 1], W.prev_vel[3 * ib + 2]);
    V3<R> pwb = v3<R>(W.prev_omega[3 * ib], W.prev_omega[3 * ib + 1], W.prev_omega[3 * ib + 2]);
    const R mud = (W.material[4 * ia + 1] + W.material[4 * ib + 1]) / (R)2.0f;
    const R e = W.material[4 * ia + 2] * W.material[4 * ib + 2];
    const R* c = W.contacts + 12 * (size_t)(W.scene_contact_cap[s] + W.pair_cstart[p]);
    for (int i = 0; i < nc; ++i) {
        const R* ci = c + 12 * i;
        Pcpd<R> pc;   // calculate_positional_constraint_preprocessed_data (the poses do not change here)
        pc.r1 = qrotate(qa, v3<R>(ci[0], ci[1], ci[2]));
        pc.r2 = qrotate(qb, v3<R>(ci[4], ci[5], ci[6]));
        pc.I1 = Ia;
        pc.I2 = Ib;
        contact_velocity<R, EXACT>(pc, a, b, ci, h, mud, e, va, wa, vb, wb, pva, pwa, pvb, pwb);
    }
    if (!a.fixed) {
        W.vel[3 * ia] = va.x; W.vel[3 * ia + 1] = va.y; W.vel[3 * ia + 2] = va.z;
        W.omega[3 * ia] = wa.x; W.omega[3 * ia + 1] = wa.y; W.omega[3 * ia + 2] = wa.z;
    }
    if (!b.fixed) {
        W.vel[3 * ib] = vb.x; W.vel[3 * ib + 1] = vb.y; W.vel[3 * ib + 2] = vb.z;
        W.omega[3 * ib] = wb.x; W.omega[3 * ib + 1] = wb.y; W.omega[3 * ib + 2] = wb.z;
    }
}

// ---------------------------------------------------------------------------------------------
// One full step of scene s by group g

// Level-by-level sweep of the Gauss–Seidel schedule. With a grid group, a run of consecutive
// levels that each hold at most SOLO_NODES nodes is swept by CTA 0 alone, separated by
// __syncthreads, while the other CTAs wait at one grid barrier: the dependent chain of small levels
// then costs a block barrier per level instead of a grid barrier. Larger levels use the whole grid.
constexpr int SOLO_NODES = 2 * BLOCK;   // default of WorldView::solo_nodes

template <typename R, bool EXACT, bool VELOCITY, class G>
__device__ void sweep_levels(const WorldView<R>& W, const G& g, int s, R hR) {
    const SchedView<R> v = sched_view(W, s, VELOCITY ? 1 : 0);
    const int L = *(volatile int*)v.levels;
    const int* lstart = v.count;
    const int solo = W.solo_nodes > 0 ? W.solo_nodes : SOLO_NODES;
    int l = 0;
    while (l < L) {
        int cnt = lstart[l + 1] - lstart[l];
        if (g.nblocks() == 1 || cnt > solo) {
            for (int i = lstart[l] + g.rank(); i < lstart[l + 1]; i += g.size()) {
                if (VELOCITY) vsolve_node<R, EXACT>(W, s, v.nodes[i], hR);
                else solve_node<R, EXACT>(W, s, v.nodes[i], hR);
            }
            g.sync();
            ++l;
            continue;
        }
        int l2 = l;
        while (l2 < L && lstart[l2 + 1] - lstart[l2] <= solo) ++l2;
        if (g.block() == 0) {
            for (int k = l; k < l2; ++k) {
                for (int i = lstart[k] + (int)threadIdx.x; i < lstart[k + 1]; i += blockDim.x) {
                    if (VELOCITY) vsolve_node<R, EXACT>(W, s, v.nodes[i], hR);
                    else solve_node<R, EXACT>(W, s, v.nodes[i], hR);
                }
                __syncthreads();
            }
        }
        g.sync();
        l = l2;
    }
}

template <typename R, bool EXACT, class G>
__device__ void step_scene(const WorldView<R>& W, const G& g, int s, const StepParams& P, NarrowSmem<R>& sm, int* smem) {
    if (!(P.dt > 0.0)) return;   // pbd.cpp:471
    const double h = P.dt / P.num_substeps;
    const R hR = (R)h;
    const int b0 = W.scene_body[s], b1 = W.scene_body[s + 1];
    const bool timer = W.phase_ns && g.rank() == 0;
    unsigned long long t_last = timer ? global_ns() : 0;
    auto mark = [&](int ph) {
        if (timer) {
            unsigned long long t = global_ns();
            atomicAdd(&W.phase_ns[ph], t - t_last);
            t_last = t;
        }
    };
    broad_phase(W, g, s, smem);
    mark(PH_BROAD);
    islands(W, g, s, P.dt);
    mark(PH_ISLANDS);
    schedule(W, g, s, smem);
    mark(PH_SCHEDULE);
    const int e0 = W.scene_ext[s], e1 = W.scene_ext[s + 1];
    for (int sub = 0; sub < P.num_substeps; ++sub) {
        for (int b = b0 + g.rank(); b < b1; b += g.size()) {
            predict_body<R, EXACT>(W, b, h);
            if constexpr (!EXACT) stage_body(W, b);
        }
        for (int e = e0 + g.rank(); e < e1; e += g.size())
            for (int k = 0; k < 4; ++k) W.ext_lambda[4 * (size_t)e + k] = 0.0;
        if (g.rank() == 0) {
            W.contact_count[s] = 0;
            W.work[s] = 0;
            if (s == 0) atomicAdd(&W.queue[4], 1);
            W.act_count[2 * s] = 0;
            W.act_count[2 * s + 1] = 0;
        }
        g.sync();
        mark(PH_PREDICT);
        if (P.enable_collisions) {
            transform_hulls<R, EXACT>(W, g, s, sub == 0);
            g.sync();
            mark(PH_TRANSFORM);
            narrowphase<R, EXACT>(W, g, s, sm);
        } else {
            const int np = min(W.pair_count[s], W.scene_pair_cap[s + 1] - W.scene_pair_cap[s]);
            for (int p = g.rank(); p < np; p += g.size()) W.pair_ccount[W.scene_pair_cap[s] + p] = 0;
        }
        g.sync();
        if constexpr (!EXACT) {   // the FP32 sweeps' per-substep solve frames (the phased form's cull writes them)
            const int np = min(W.pair_count[s], W.scene_pair_cap[s + 1] - W.scene_pair_cap[s]);
            const int pb = W.scene_pair_cap[s];
            for (int p = g.rank(); p < np; p += g.size()) {
                const int2 pr = W.pairs[pb + p];
                W.pair_base[pb + p] = fbase4(W, pr.x, pr.y);
            }
            for (int e = e0 + g.rank(); e < e1; e += g.size()) W.ext_base[e] = fbase4(W, W.ext[e].e1, W.ext[e].e2);
            g.sync();
        }
        mark(PH_NARROW);
        resched(W, g, s);
        mark(PH_SCHEDULE);
        for (int it = 0; it < P.num_pos_iters; ++it) sweep_levels<R, EXACT, false>(W, g, s, hR);
        mark(PH_SOLVE);
        for (int b = b0 + g.rank(); b < b1; b += g.size()) {
            if constexpr (!EXACT) fold_body(W, b);
            velocity_body<R, EXACT>(W, b, h);
        }
        g.sync();
        mark(PH_VELOCITY);
        sweep_levels<R, EXACT, true>(W, g, s, hR);
        mark(PH_VSOLVE);
    }
}

template <typename R, bool EXACT>
__global__ void __launch_bounds__(BLOCK, 1) step_kernel_cta(WorldView<R> W, StepParams P) {
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    __shared__ int scan_smem[32];
    NarrowSmem<R>* sms = reinterpret_cast<NarrowSmem<R>*>(dyn_smem);
    NarrowSmem<R>& sm = sms[threadIdx.x >> 5];
    CtaGroup g;
    for (int s = blockIdx.x; s < W.num_scenes; s += gridDim.x) {
        step_scene<R, EXACT>(W, g, s, P, sm, scan_smem);
        __syncthreads();
    }
}

template <typename R, bool EXACT>
__global__ void __launch_bounds__(BLOCK, 1) step_kernel_grid(WorldView<R> W, StepParams P) {
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    __shared__ int scan_smem[32];
    NarrowSmem<R>* sms = reinterpret_cast<NarrowSmem<R>*>(dyn_smem);
    NarrowSmem<R>& sm = sms[threadIdx.x >> 5];
    if (frame_abandoned(W.status)) return;
    GridGroup g;
    g.bar = W.barrier;
    g.status = W.status;
    g.limit_ns = W.wait_ns;
    step_scene<R, EXACT>(W, g, 0, P, sm, scan_smem);
}

}  // namespace rp
