// k_batch1.cu -- a whole batch of grids in ONE persistent launch over device
// work queues (no counterpart in the reference, which sweeps one grid per
// process with one launch per sweep: src/stencil_dispatch.cu:153-157).
//
// One cooperative launch holds every CTA the device can keep resident (one
// per SM).  The CTAs form teams; a team sweeps one grid at a time, all of
// its sweeps, with a bounded barrier over the team's CTAs between sweeps
// (a counter in global memory, as the persistent single-grid kernels use over
// the whole GPU), then takes the next grid.  3-D grids are swept by the
// stream kernel's per-CTA code (stream_body.cuh: TMA plane ring, z register
// queue; tensor maps per grid in the workspace), 2-D grids by the rows
// kernel's (rows_body.cuh: register-queue chunk columns).  Every cell keeps
// the reference's summation order and division, so results are bit-identical
// to the ping-pong loop.
//
// Teams and tiers.  The host puts each grid in a tier by the team size its
// cells keep busy (about STENCIL_BATCH1_CELLS_PER_CTA_{2D,3D} update cells
// per CTA per sweep, so the per-sweep barrier stays a small share), or by the
// job's own team field (an autotuner's choice); tier t has
// a nominal team size and a queue of its grids, largest work first.  All
// CTAs start in the first tier as teams of its size; a team whose tier queue
// is empty splits into the next tier's teams (its own CTAs: never waiting on
// another team) and takes grids from that queue.  Large grids therefore run
// first on large teams and the small ones fill the end on small teams.  A
// team's leader takes the next grid with an atomic on the tier's queue and
// passes its index to the team through a mailbox word read after a team
// barrier.
//
// Grids whose rows are not 16-byte aligned (nx % 4 != 0) are swept in
// pitched copies in the workspace, copied in by the team before the first
// sweep and back after the last (inside the same launch).  Every wait is
// bounded; a team that gives up sets an abort word, after which no team takes
// another grid.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "host.hpp"
#include "rows_body.cuh"
#include "stream_body.cuh"

namespace st {
namespace {

// Stream shapes of the batch kernel per radius: the persistent single-grid
// defaults (one row per thread at R = 1, 3, 4; two rows per thread at R = 2)
// with 15 consumer warps instead of 16 (tiles of 15 or 30 rows), so that the
// block is 16 warps: four per SM sub-partition leave 128 registers a thread
// (17 warps would leave 96, too few for the code of every radius in one
// kernel without spills).
// N: narrow tiles (64 x 30) for grids at most 64 cells wide at R <= 2, where
// a 128-wide tile would leave most consumer threads without cells.
template <int R, bool N = false> struct B1S;
template <> struct B1S<1, false> { static constexpr int TX = 128, TY = 15, RY = 1, NS = 16; };
template <> struct B1S<2, false> { static constexpr int TX = 128, TY = 30, RY = 2, NS = 8; };
template <> struct B1S<3, false> { static constexpr int TX = 128, TY = 15, RY = 1, NS = 8; };
template <> struct B1S<4, false> { static constexpr int TX = 128, TY = 15, RY = 1, NS = 8; };
template <> struct B1S<1, true> { static constexpr int TX = 64, TY = 30, RY = 1, NS = 16; };
template <> struct B1S<2, true> { static constexpr int TX = 64, TY = 30, RY = 1, NS = 16; };
template <int R, bool N = false>
using B1Shape = StreamShape<R, B1S<R, N>::TX, B1S<R, N>::TY, B1S<R, N>::RY, B1S<R, N>::NS>;

constexpr int kB1Threads = 512;
static_assert(B1Shape<1>::THREADS == kB1Threads && B1Shape<2>::THREADS == kB1Threads &&
                  B1Shape<3>::THREADS == kB1Threads && B1Shape<4>::THREADS == kB1Threads &&
                  B1Shape<1, true>::THREADS == kB1Threads && B1Shape<2, true>::THREADS == kB1Threads,
              "every stream shape of the batch kernel has the kernel's block size");
constexpr int kB1MaxSlots = 16;   // mbarriers: full[16], empty[16], swept
constexpr int kB1BarBytes = 384;  // (2 * 16 + 1) * 8 rounded up to 128
template <int R, bool N = false>
constexpr int b1_ring_bytes() { return B1S<R, N>::NS * B1Shape<R, N>::SLOT_FLOATS * 4; }
constexpr int kB1RingBytes =
    std::max(std::max(std::max(b1_ring_bytes<1>(), b1_ring_bytes<2>()), std::max(b1_ring_bytes<3>(), b1_ring_bytes<4>())),
             std::max(b1_ring_bytes<1, true>(), b1_ring_bytes<2, true>()));
constexpr int kB1Smem = 128 + kB1BarBytes + kB1RingBytes;
static_assert(B1S<1>::NS <= kB1MaxSlots && B1S<2>::NS <= kB1MaxSlots && B1S<1, true>::NS <= kB1MaxSlots &&
                  B1S<2, true>::NS <= kB1MaxSlots,
              "ring fits the mbarrier area");

// 2-D grids read with plain (L1-cached) loads: every read of another CTA's
// writes follows the team barrier's acquire and a CTA barrier (GB300, the
// 512-grid benchmark batch: its 2-D grids from 640^2 up 0.94 -> 0.82 s, those
// below 0.154 -> 0.122 s, against ld.global.cg).  0 selects ld.global.cg.
#ifndef STENCIL_B1_ROWS_L1
#define STENCIL_B1_ROWS_L1 1
#endif

constexpr int kB1MaxTiers = 12;
constexpr int kB1MaxCtas = 1024;
constexpr unsigned kB1Stop = 0xffffffffu;

// One grid as the batch kernel sweeps it.
struct B1Job {
    float *a, *b;          // the buffers swept (a: initial state); pitched copies when staged
    float *ua, *ub;        // the caller's buffers of a staged grid, else null
    Geom g;                // g.sy: row pitch of a and b (a multiple of 4)
    int dims, iters;
    int map_pair;          // 3-D: its tensor maps (a, b) are maps[2 * map_pair] and the next, else -1
    int narrow;            // 3-D: swept with the narrow tiles of its radius
    int tiles_x, tiles_y, zchunk, items;  // 3-D work items for its tier's team size
    int hb, nblk;          // 2-D row blocks for its tier's team size
    long long rows;        // rows of the grid (ny * nz)
};

struct B1Tier {
    int team;   // nominal team size (CTAs)
    int first;  // first job of the tier in the job table
    int njobs;
    int pad;
};

struct B1Args {
    const B1Job *jobs;
    const CUtensorMap *maps;
    unsigned *ctr;  // queues [kB1MaxTiers]; team counters, mailboxes, sweep counters [kB1MaxTiers][G] each; abort word
    int ntiers;
    int njobs;
    int nmaps;      // entries of maps (two per 3-D job)
    int pad;
    B1Tier tier[kB1MaxTiers];
};

__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ unsigned ld_volatile_u32(const unsigned *p) {
    return *reinterpret_cast<const volatile unsigned *>(p);
}

// The part of the team of `size` CTAs starting at *start (this CTA among
// them) that forms this CTA's team of nominal size k: consecutive teams of k
// CTAs, the last one also taking the remainder.
__device__ __forceinline__ void team_split(unsigned *start, unsigned *size, int k, unsigned cta) {
    const unsigned kk = (unsigned)max(1, k);
    const unsigned n = max(1u, *size / kk);
    const unsigned idx = min((cta - *start) / kk, n - 1);
    *start += idx * kk;
    *size = idx == n - 1 ? *size - idx * kk : kk;
}

// Copies a staged grid's two buffers between the caller's rows (pitch nx)
// and the pitched copies (pitch g.sy): in = to the copies.  A warp per row,
// rows spread over the team; four loads per lane in flight.
__device__ __forceinline__ void stage_rows(const B1Job &J, bool in, unsigned rel, unsigned size) {
    const int lane = threadIdx.x & 31;
    const long long nwarps = (long long)size * (kB1Threads / 32);
    const int nx = J.g.nx;
    const long long px = J.g.sy;
    for (long long r = (long long)rel * (kB1Threads / 32) + (threadIdx.x >> 5); r < J.rows; r += nwarps) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const float *src = in ? (h ? J.ub : J.ua) + r * nx : (h ? J.b : J.a) + r * px;
            float *dst = in ? (h ? J.b : J.a) + r * px : (h ? J.ub : J.ua) + r * nx;
            for (int x = lane; x < nx; x += 128) {
                float v[4];
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (x + 32 * k < nx) v[k] = in ? __ldcs(src + x + 32 * k) : __ldcg(src + x + 32 * k);
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (x + 32 * k < nx) dst[x + 32 * k] = v[k];
            }
        }
    }
}

// Where a CTA is in the batch: its tier, its team (first CTA, size; this
// CTA's rank in it), the values the team's two counters of this tier hold
// after its last barrier (cnt: barriers of all its CTAs -- job hand-out,
// copies, end of a grid; scnt: the sweep barriers of 3-D grids, which only
// the CTAs with work items join), the current job and the ring's initialised
// slots.  Kept in shared memory and changed by thread 0 only
// (before a CTA barrier), so that no register holds it across a grid's
// sweeps.
struct B1Ctl {
    int t;
    unsigned start, size, rel, cnt, scnt;
    unsigned job;
    int prev_ns;
    int ok;
};

__device__ __forceinline__ unsigned *team_counter(const B1Args &A, const B1Ctl &c) {
    return A.ctr + kB1MaxTiers + c.t * gridDim.x + c.start;
}
__device__ __forceinline__ unsigned *sweep_counter(const B1Args &A, const B1Ctl &c) {
    return team_counter(A, c) + 2 * kB1MaxTiers * gridDim.x;
}
__device__ __forceinline__ unsigned *abort_word(const B1Args &A) {
    return A.ctr + kB1MaxTiers * (1 + 3 * gridDim.x);
}

// Barrier over the team's CTAs: this CTA's stores first (CTA barrier), then
// thread 0 arrives and waits (bounded) until the counter reaches the next
// multiple of the team size.
__device__ __forceinline__ bool team_barrier(const B1Args &A, B1Ctl &c) {
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned *bar = team_counter(A, c);
        grid_arrive(bar);
        c.cnt += c.size;
        c.ok = grid_wait_bounded(bar, c.cnt) ? 1 : 0;
    }
    __syncthreads();
    return c.ok != 0;
}

// Thread 0: the team's next job, moving on to the next tier (its team split
// into that tier's teams) while the current one has none left.  Sets c.job
// to the job's index in the job table, or kB1Stop once every tier is done or
// a wait gave up or another team aborted.
__device__ __forceinline__ void next_job(const B1Args &A, B1Ctl &c) {
    unsigned *abort_at = abort_word(A);
    for (;;) {
        if (c.t < 0 || c.job == kB1Stop) {
            if (++c.t >= A.ntiers) { c.job = kB1Stop; return; }
            team_split(&c.start, &c.size, A.tier[c.t].team, blockIdx.x);
            c.rel = blockIdx.x - c.start;
            c.cnt = c.scnt = 0;
        }
        unsigned *bar = team_counter(A, c);
        unsigned *box = bar + kB1MaxTiers * gridDim.x;  // the team's mailbox
        if (c.rel == 0) {
            const unsigned j = ld_volatile_u32(abort_at) ? kB1Stop - 1 : atomicAdd(&A.ctr[c.t], 1u);
            *reinterpret_cast<volatile unsigned *>(box) = j;
        }
        grid_arrive(bar);
        c.cnt += c.size;
        if (!grid_wait_bounded(bar, c.cnt)) { c.job = kB1Stop; c.t = A.ntiers; return; }
        const unsigned j = ld_volatile_u32(box);
        if (j == kB1Stop - 1) { c.job = kB1Stop; c.t = A.ntiers; return; }
        const B1Tier T = A.tier[c.t];
        if (j < (unsigned)T.njobs) {
            c.job = (unsigned)T.first + j;
            // the table's own consistency (checked by the host too): a job
            // in range, a 3-D job's two tensor maps in the map table
            const B1Job *J = A.jobs + c.job;
            if (c.job >= (unsigned)A.njobs ||
                (J->dims == 3 && (J->map_pair < 0 || 2 * J->map_pair + 1 >= A.nmaps))) {
                report_status(kStatusBadLaunch);
                atomicExch(abort_at, 1u);
                c.job = kB1Stop;
                c.t = A.ntiers;
            }
            return;
        }
        c.job = kB1Stop;  // this tier is done: next tier
    }
}

// All sweeps of a 3-D grid on the team (stream code; the producer warp
// waits on the team's sweep counter between sweeps).  Only the first
// min(items, team size) CTAs of the team take part, and the sweep counter is
// theirs alone: the stream code's consumers wait for nothing but their own
// planes, so a CTA without a work item would arrive for every sweep at once
// -- and the idle CTAs go on to the end-of-grid barrier at once -- and either
// would let the others' producers pass a sweep barrier early.  The ring's mbarriers are set up afresh for the
// grid's shape (those of the previous grid, all of whose phases completed
// before the CTA barrier that ended it, are invalidated first).
template <int R, bool N>
__device__ __forceinline__ void job3d(const B1Args &A, const B1Job *__restrict__ J, unsigned char *base,
                                      B1Ctl &c) {
    using Sh = B1S<R, N>;
    using S = B1Shape<R, N>;
    const unsigned P = min((unsigned)J->items, c.size);
    __syncthreads();
    if (c.rel < P) {
        uint64_t *full = reinterpret_cast<uint64_t *>(base);
        uint64_t *empty = full + kB1MaxSlots;
        uint64_t *swept = empty + kB1MaxSlots;
        float *ring = reinterpret_cast<float *>(base + kB1BarBytes);
        const CUtensorMap *m0 = A.maps + 2 * J->map_pair, *m1 = m0 + 1;
        if (threadIdx.x == 0) {
            const int prev = c.prev_ns;
            if (prev) {
                for (int s = 0; s < prev; ++s) {
                    mbar_inval(&full[s]);
                    mbar_inval(&empty[s]);
                }
                mbar_inval(swept);
            }
            for (int s = 0; s < Sh::NS; ++s) {
                mbar_init(&full[s], 1);
                mbar_init(&empty[s], S::CWARPS);
            }
            mbar_init(swept, S::CWARPS);
            fence_mbar_init();
            prefetch_tensormap(m0);
            prefetch_tensormap(m1);
            c.prev_ns = Sh::NS;
        }
        __syncthreads();
        stream3d_sweeps<R, Sh::TX, Sh::TY, Sh::RY, Sh::NS, true, false>(
            ring, full, empty, swept, m0, m1, J->b, J->a, J->g, J->tiles_x, J->tiles_y, J->zchunk,
            J->items, J->iters, sweep_counter(A, c), c.scnt, c.rel, P, true);
    }
    __syncthreads();
    if (threadIdx.x == 0) c.scnt += (unsigned)(J->iters - 1) * P;
}

// All sweeps of a 2-D grid on the team.
template <int R>
__device__ __forceinline__ bool job2d(const B1Args &A, const B1Job *__restrict__ J, B1Ctl &c) {
    const int iters = J->iters;
    for (int sw = 0; sw < iters; ++sw) {
        const float *src = (sw & 1) ? J->b : J->a;
        float *dst = (sw & 1) ? J->a : J->b;
        rows2d_sweep_d<R, kB1Threads, (R == 1 ? 4 : R == 2 ? 2 : 1), STENCIL_B1_ROWS_L1 != 0>(
            src, dst, J->g, J->hb, J->nblk, c.rel, c.size);
        if (sw + 1 < iters && !team_barrier(A, c)) return false;
    }
    return true;
}

// One grid on the team: copies in, sweeps, a team barrier, copies out.
__device__ __forceinline__ bool run_job(const B1Args &A, const B1Job *__restrict__ J,
                                        unsigned char *base, B1Ctl &c) {
    // A grid with no sweep still ends with a team barrier: the leader's next
    // mailbox write must follow every member's read of this grid's index.
    if (J->iters <= 0) return team_barrier(A, c);
    if (J->ua) {
        stage_rows(*J, true, c.rel, c.size);
        if (!team_barrier(A, c)) return false;
    }
    if (J->dims == 3) {
        switch (J->g.radius * 2 + (J->narrow ? 1 : 0)) {
            case 2: job3d<1, false>(A, J, base, c); break;
            case 3: job3d<1, true>(A, J, base, c); break;
            case 4: job3d<2, false>(A, J, base, c); break;
            case 5: job3d<2, true>(A, J, base, c); break;
            case 6: job3d<3, false>(A, J, base, c); break;
            default: job3d<4, false>(A, J, base, c); break;
        }
    } else {
        bool ok;
        switch (J->g.radius) {
            case 1: ok = job2d<1>(A, J, c); break;
            case 2: ok = job2d<2>(A, J, c); break;
            case 3: ok = job2d<3>(A, J, c); break;
            default: ok = job2d<4>(A, J, c); break;
        }
        if (!ok) return false;
    }
    // every CTA's last sweep stored before the copies out and the next grid
    if (!team_barrier(A, c)) return false;
    if (J->ua) stage_rows(*J, false, c.rel, c.size);
    return true;
}

__global__ void __launch_bounds__(kB1Threads, 1) k_batch1(const __grid_constant__ B1Args A) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~static_cast<uintptr_t>(127));
    __shared__ B1Ctl c;
    if (threadIdx.x == 0) {
        c.t = -1;
        c.start = 0;
        c.size = gridDim.x;
        c.rel = c.cnt = c.scnt = 0;
        c.job = kB1Stop;
        c.prev_ns = 0;
        c.ok = 1;
    }
    for (;;) {
        __syncthreads();  // every thread has read c.job (and the previous grid is done)
        if (threadIdx.x == 0) next_job(A, c);
        __syncthreads();
        if (c.job == kB1Stop) return;
        if (!run_job(A, A.jobs + c.job, base, c)) {
            if (threadIdx.x == 0) atomicExch(abort_word(A), 1u);
            return;
        }
    }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
struct B1Plan {
    B1Args args;
    size_t ctr_off = 0, ctr_bytes = 0;
    int grid = 0;
    int njobs = 0;
};

std::mutex g_b1_mu;
std::vector<std::pair<const void *, B1Plan>> g_b1;

size_t round256(size_t n) { return (n + 255) & ~(size_t)255; }

// Bytes of one pitched copy of a grid whose nx is not a multiple of 4.
size_t b1_staged_bytes(const stencil_batch_job &b) {
    if (b.nx % 4 == 0 || b.nx <= 0 || b.ny <= 0) return 0;
    const size_t px = ((size_t)b.nx + 3) & ~(size_t)3;
    const size_t rows = (size_t)b.ny * (b.dims == 3 && b.nz > 0 ? (size_t)b.nz : 1);
    return round256(px * rows * sizeof(float));
}

size_t b1_ctr_bytes(int grid) {
    return ((size_t)kB1MaxTiers * (1 + 3 * (size_t)grid) + 1) * sizeof(unsigned);
}

// Resident CTAs of the batch kernel (its shared-memory limit set once per
// device).
int b1_resident(int *grid) {
    static std::mutex mu;
    static std::vector<std::pair<int, int>> cache;
    const int dev = current_device();
    std::lock_guard<std::mutex> lock(mu);
    for (auto &c : cache)
        if (c.first == dev) { *grid = c.second; return STENCIL_OK; }
    const void *fn = reinterpret_cast<const void *>(k_batch1);
    ST_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kB1Smem));
    int per_sm = 0;
    ST_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kB1Threads, kB1Smem));
    const int n = std::min(kB1MaxCtas, per_sm * num_sms());
    if (n < 1) return fail(STENCIL_EUNSUPPORTED, "the batch kernel does not fit on an SM");
    cache.push_back({dev, n});
    *grid = n;
    return STENCIL_OK;
}

long long env_ll(const char *name, long long dflt) {
    const char *e = std::getenv(name);
    if (e && *e) {
        char *end = nullptr;
        const long long v = std::strtoll(e, &end, 10);
        if (end && *end == 0 && v > 0) return v;
    }
    return dflt;
}

}  // namespace

// Update cells per CTA per sweep that a team keeps, and the largest team
// (environment variables of the same names override them at prepare time).
// GB300, the 512-grid benchmark batch, seconds per batch for 2-D / 3-D
// cells per CTA: 25k/50k 2.79, 50k/50k 2.76, 50k/100k 2.90, 100k/100k 3.06,
// 100k/200k 3.36 (before the L1-cached 2-D loads; with them 50k/50k 2.63).
#ifndef STENCIL_BATCH1_CELLS_PER_CTA_2D
#define STENCIL_BATCH1_CELLS_PER_CTA_2D 50000
#endif
#ifndef STENCIL_BATCH1_CELLS_PER_CTA_3D
#define STENCIL_BATCH1_CELLS_PER_CTA_3D 50000
#endif

size_t batch1_bytes_for(const stencil_batch_job *jobs, int njobs) {
    int n3 = 0;
    size_t copies = 0;
    for (int i = 0; i < njobs; ++i) {
        n3 += jobs[i].dims == 3;
        copies += 2 * b1_staged_bytes(jobs[i]);
    }
    return round256((size_t)njobs * sizeof(B1Job)) + round256((size_t)n3 * 2 * sizeof(CUtensorMap)) +
           round256(b1_ctr_bytes(kB1MaxCtas)) + copies;
}

// Validated jobs -> job table, tensor maps and tiers in the workspace.
int batch1_prepare(const stencil_batch_job *jobs, int njobs, void *d_workspace,
                   size_t workspace_bytes, cudaStream_t s) {
    // every job checked before anything reaches the device
    for (int i = 0; i < njobs; ++i) {
        stencil_params p;
        const int rc = check_batch_job(jobs[i], i, &p);
        if (rc) return rc;
    }
    if (workspace_bytes < batch1_bytes_for(jobs, njobs))
        return fail(STENCIL_EINVAL, "workspace too small: %zu < %zu bytes (stencil_batch_workspace_bytes_for)",
                    workspace_bytes, batch1_bytes_for(jobs, njobs));
    int grid = 0;
    int rc = b1_resident(&grid);
    if (rc) return rc;
    char *ws = static_cast<char *>(d_workspace);
    int n3 = 0;
    for (int i = 0; i < njobs; ++i) n3 += jobs[i].dims == 3;
    const size_t maps_off = round256((size_t)njobs * sizeof(B1Job));
    const size_t ctr_off = maps_off + round256((size_t)n3 * 2 * sizeof(CUtensorMap));
    size_t copy_off = ctr_off + round256(b1_ctr_bytes(kB1MaxCtas));

    // Team sizes: G, G/2, G/4, ... 1; a grid's tier is the largest of them
    // at most its cells / cells-per-CTA (and at most the largest team).
    std::vector<int> ladder;
    for (int k = grid; k >= 1; k /= 2) ladder.push_back(k);
    const long long cpc2 = env_ll("STENCIL_BATCH1_CELLS_PER_CTA_2D", STENCIL_BATCH1_CELLS_PER_CTA_2D);
    const long long cpc3 = env_ll("STENCIL_BATCH1_CELLS_PER_CTA_3D", STENCIL_BATCH1_CELLS_PER_CTA_3D);
    const long long kmax = env_ll("STENCIL_BATCH1_MAX_TEAM", std::max(1, grid / 4));

    std::vector<B1Job> table(njobs);
    std::vector<int> tier_of(njobs);
    std::vector<double> work(njobs);
    std::vector<CUtensorMap> maps;
    maps.reserve(2 * n3);
    for (int i = 0; i < njobs; ++i) {
        const stencil_batch_job &b = jobs[i];
        stencil_params p;
        rc = check_batch_job(b, i, &p);
        if (rc) return rc;
        Geom g = make_geom(p);
        B1Job &J = table[i];
        J = B1Job{};
        J.a = b.d_u1;
        J.b = b.d_u2;
        J.dims = p.dims;
        J.iters = b.iterations;
        J.map_pair = -1;
        J.rows = (long long)p.ny * (p.dims == 3 ? p.nz : 1);
        const size_t sb = b1_staged_bytes(b);
        if (sb) {
            J.ua = b.d_u1;
            J.ub = b.d_u2;
            J.a = reinterpret_cast<float *>(ws + copy_off);
            J.b = reinterpret_cast<float *>(ws + copy_off + sb);
            copy_off += 2 * sb;
            const long long px = ((long long)b.nx + 3) & ~3LL;
            g.sy = px;
            g.sz = px * b.ny;
        }
        J.g = g;
        const long long cells = (long long)(p.nx - 2 * p.radius) * (p.ny - 2 * p.radius) *
                                (p.dims == 3 ? p.nz - 2 * p.radius : 1);
        // the job's own team size (a tuner's choice), else from its cells
        const long long want =
            b.team > 0 ? std::min<long long>(b.team, grid)
                       : std::max(1LL, std::min(kmax, cells / (p.dims == 3 ? cpc3 : cpc2)));
        int t = 0;
        while (ladder[t] > want) ++t;
        tier_of[i] = t;
        work[i] = (double)cells * b.iterations;
        const int team = ladder[t];
        if (p.dims == 3) {
            int tx = 0, ty = 0;
            J.narrow = p.radius <= 2 && p.nx <= 64;
            switch (p.radius * 2 + J.narrow) {
                case 2: tx = B1S<1>::TX; ty = B1S<1>::TY; break;
                case 3: tx = B1S<1, true>::TX; ty = B1S<1, true>::TY; break;
                case 4: tx = B1S<2>::TX; ty = B1S<2>::TY; break;
                case 5: tx = B1S<2, true>::TX; ty = B1S<2, true>::TY; break;
                case 6: tx = B1S<3>::TX; ty = B1S<3>::TY; break;
                default: tx = B1S<4>::TX; ty = B1S<4>::TY; break;
            }
            stream3d_plan(g, tx, ty, team, &J.tiles_x, &J.tiles_y, &J.zchunk, &J.items);
            CUtensorMap m[2];
            const long long dims[3] = {g.nx, g.ny, g.nz};
            const int box[3] = {tx + 2 * ((p.radius + 3) & ~3), ty + 2 * p.radius, 1};
            rc = make_tensor_map(&m[0], J.a, 3, dims, box, g.sy, true);
            if (!rc) rc = make_tensor_map(&m[1], J.b, 3, dims, box, g.sy, true);
            if (rc) return rc;
            J.map_pair = (int)(maps.size() / 2);
            maps.push_back(m[0]);
            maps.push_back(m[1]);
        } else {
            if ((long long)(g.sy / 4) * (g.ny - 2 * g.radius) >= (1LL << 31))
                return fail(STENCIL_EUNSUPPORTED, "job %d: 2-D grid of 2^31 or more chunk-rows", i);
            rows2d_plan(g, (long long)team * kB1Threads, &J.hb, &J.nblk);
        }
    }
    // job table: by tier, then largest work first
    std::vector<int> order(njobs);
    for (int i = 0; i < njobs; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return tier_of[x] != tier_of[y] ? tier_of[x] < tier_of[y] : work[x] > work[y];
    });
    std::vector<B1Job> sorted(njobs);
    B1Plan plan;
    B1Args &A = plan.args;
    A = B1Args{};
    for (int k = 0; k < njobs; ++k) {
        const int i = order[k];
        sorted[k] = table[i];
        const int t = tier_of[i];
        if (A.ntiers == 0 || A.tier[A.ntiers - 1].team != ladder[t]) {
            if (A.ntiers == kB1MaxTiers) return fail(STENCIL_EUNSUPPORTED, "too many tiers");
            A.tier[A.ntiers] = B1Tier{ladder[t], k, 0, 0};
            ++A.ntiers;
        }
        ++A.tier[A.ntiers - 1].njobs;
    }
    // every 3-D job has its own map pair; 2-D jobs none
    {
        std::vector<char> seen(maps.size() / 2, 0);
        for (const B1Job &J : sorted) {
            if (J.dims != 3) {
                if (J.map_pair != -1) return fail(STENCIL_EINVAL, "internal: 2-D job with tensor maps");
                continue;
            }
            if (J.map_pair < 0 || J.map_pair >= (int)seen.size() || seen[J.map_pair]++)
                return fail(STENCIL_EINVAL, "internal: tensor-map table does not match the jobs");
        }
    }
    A.njobs = njobs;
    A.nmaps = (int)maps.size();
    A.jobs = reinterpret_cast<const B1Job *>(ws);
    A.maps = reinterpret_cast<const CUtensorMap *>(ws + maps_off);
    A.ctr = reinterpret_cast<unsigned *>(ws + ctr_off);
    plan.ctr_off = ctr_off;
    plan.ctr_bytes = b1_ctr_bytes(grid);
    plan.grid = grid;
    plan.njobs = njobs;
    if (njobs) ST_CUDA(cudaMemcpyAsync(ws, sorted.data(), njobs * sizeof(B1Job), cudaMemcpyHostToDevice, s));
    if (!maps.empty())
        ST_CUDA(cudaMemcpyAsync(ws + maps_off, maps.data(), maps.size() * sizeof(CUtensorMap),
                                cudaMemcpyHostToDevice, s));
    ST_CUDA(cudaStreamSynchronize(s));
    std::lock_guard<std::mutex> lock(g_b1_mu);
    for (auto &c : g_b1)
        if (c.first == d_workspace) { c.second = plan; return STENCIL_OK; }
    g_b1.emplace_back(d_workspace, plan);
    return STENCIL_OK;
}

namespace {
bool b1_recall(const void *ws, B1Plan *plan) {
    std::lock_guard<std::mutex> lock(g_b1_mu);
    for (auto &c : g_b1)
        if (c.first == ws) { *plan = c.second; return true; }
    return false;
}
}  // namespace

bool batch1_known(const void *ws) {
    B1Plan p;
    return b1_recall(ws, &p);
}

// One memset node (queues, team and sweep counters, mailboxes, abort word) and the
// kernel.
int batch1_launch(const void *d_workspace, cudaStream_t s) {
    B1Plan plan;
    if (!b1_recall(d_workspace, &plan)) return fail(STENCIL_EINVAL, "not a one-launch batch workspace");
    note_launches("batch-one-launch", plan.njobs ? 1 : 0);
    if (!plan.njobs) return STENCIL_OK;
    ST_CUDA(cudaMemsetAsync(static_cast<char *>(const_cast<void *>(d_workspace)) + plan.ctr_off, 0,
                            plan.ctr_bytes, s));
    void *args[] = {&plan.args};
    ST_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(k_batch1), dim3(plan.grid),
                                        dim3(kB1Threads), args, kB1Smem, s));
    return STENCIL_OK;
}

int batch1_launches(const void *d_workspace) {
    B1Plan plan;
    return b1_recall(d_workspace, &plan) && plan.njobs ? 1 : 0;
}

int batch1_teams(const void *d_workspace, int *ntiers, int *team_sizes, int *tier_jobs, int max_tiers) {
    B1Plan plan;
    if (!b1_recall(d_workspace, &plan)) return fail(STENCIL_EINVAL, "not a one-launch batch workspace");
    *ntiers = plan.args.ntiers;
    for (int t = 0; t < plan.args.ntiers && t < max_tiers; ++t) {
        if (team_sizes) team_sizes[t] = plan.args.tier[t].team;
        if (tier_jobs) tier_jobs[t] = plan.args.tier[t].njobs;
    }
    return STENCIL_OK;
}

void batch1_forget(const void *d_workspace) {
    std::lock_guard<std::mutex> lock(g_b1_mu);
    for (size_t i = 0; i < g_b1.size(); ++i)
        if (g_b1[i].first == d_workspace) {
            g_b1.erase(g_b1.begin() + i);
            return;
        }
}

}  // namespace st
