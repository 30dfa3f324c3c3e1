// List rebuild path of the GB300 DEM engine: Morton keys, stable LSB radix
// sort, particle reorder, cell ranges, Verlet lists, wall mesh tree and wall lists.
//
// Reference counterparts (gpudem): dk_morton_key / update_pList_withSort
// (BoundingBox.cu:1007, :664), radixSortUint32 / CUB SortPairs
// (BoundingBox.cu:33, :1235), d_swap_ps (BoundingBox.cu:928), d_update_pList
// (BoundingBox.cu:1266), k_update_neighborlist_endsort (BoundingBox.cu:1106),
// buildBVH (BVH.cu:741), k_update_neighborlist_wall (BVH.cu:493).
//
// Every kernel that decides list membership uses the reference's FP64
// arithmetic in the same operation order; this file is compiled with
// -fmad=false so no multiply-add is contracted.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gdem_internal.cuh"

namespace gdem {

// ===================================================================== radix sort
// Stable least-significant-digit radix sort of (key, value) pairs with 8-bit
// digits.  One pass = upsweep (per-tile digit histograms, digit-major table),
// scan (per-digit exclusive scan over tiles), downsweep (stable scatter).  The
// scatter ranks equal digits inside a tile with __match_any_sync, so the
// permutation is the unique stable one — the same that radixSortUint32
// (BoundingBox.cu:33-104) and CUB's SortPairs produce.  No kernel waits on
// another block.
constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;

int rs_blocks_for(int n) { return n <= 0 ? 1 : (n + RS_TILE - 1) / RS_TILE; }

__global__ void __launch_bounds__(RS_THREADS) k_rs_upsweep(const uint32_t* __restrict__ keys, int n,
                                                           int shift, uint32_t* __restrict__ hist,
                                                           int nblocks, const Ctl* ctl, int gated) {
    if (gated && ctl->refresh == 0u) return;
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * RS_TILE;
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; r++) {
        const int i = base + r * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nblocks + blockIdx.x] = cnt[threadIdx.x];
}

// one block per digit: exclusive scan of that digit's tile counts
__global__ void __launch_bounds__(1024) k_rs_scan(uint32_t* __restrict__ hist, int nblocks,
                                                  uint32_t* __restrict__ tot, const Ctl* ctl, int gated) {
    if (gated && ctl->refresh == 0u) return;
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry;
    uint32_t* row = hist + (size_t)blockIdx.x * nblocks;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nblocks; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const uint32_t x = i < nblocks ? row[i] : 0u;
        uint32_t incl = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warp_sums[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const int nw = blockDim.x >> 5;
            uint32_t s = lane < nw ? warp_sums[lane] : 0u;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            if (lane < nw) warp_sums[lane] = s;  // inclusive warp prefix
        }
        __syncthreads();
        const uint32_t warp_excl = warp ? warp_sums[warp - 1] : 0u;
        const uint32_t c = carry;
        if (i < nblocks) row[i] = c + warp_excl + incl - x;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = c + warp_excl + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) tot[blockIdx.x] = carry;
}

// SMALL: few tiles (nblocks <= RS_SMALL_TILES); the tile counts are then
// read unscanned and each block sums what it needs itself, with no scan
// kernel in between.
constexpr int RS_SMALL_TILES = 32;

template <bool SMALL>
__global__ void __launch_bounds__(RS_THREADS) k_rs_downsweep(
    const uint32_t* __restrict__ kin, const int* __restrict__ vin, uint32_t* __restrict__ kout,
    int* __restrict__ vout, int n, int shift, const uint32_t* __restrict__ hist,
    const uint32_t* __restrict__ tot, int nblocks, const Ctl* ctl, int gated) {
    if (gated && ctl->refresh == 0u) return;
    constexpr int NW = RS_THREADS / 32;
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcnt[NW][256];
    __shared__ uint32_t scan_tmp[256];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    // digit base = exclusive prefix of the digit totals + this tile's offset
    uint32_t total, mine;
    if (SMALL) {
        total = 0u;
        mine = 0u;
        for (int b = 0; b < nblocks; b++) {
            const uint32_t c = hist[t * nblocks + b];
            if (b < (int)blockIdx.x) mine += c;
            total += c;
        }
    } else {
        total = tot[t];
        mine = hist[t * nblocks + blockIdx.x];
    }
    scan_tmp[t] = total;
    __syncthreads();
    for (int o = 1; o < 256; o <<= 1) {
        const uint32_t y = t >= o ? scan_tmp[t - o] : 0u;
        __syncthreads();
        scan_tmp[t] += y;
        __syncthreads();
    }
    base[t] = scan_tmp[t] - total + mine;
#pragma unroll
    for (int w = 0; w < NW; w++) wcnt[w][t] = 0;
    __syncthreads();
    const unsigned lt_mask = (1u << lane) - 1u;
    const int tile = blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ROUNDS; r++) {
        const int i = tile + r * RS_THREADS + t;
        const bool valid = i < n;
        uint32_t key = 0;
        int val = 0;
        uint32_t d = 256u;  // invalid lanes get a digit of their own
        if (valid) {
            key = kin[i];
            val = vin[i];
            d = (key >> shift) & 0xFFu;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const uint32_t wrank = __popc(peers & lt_mask);
        if (valid && (peers & lt_mask) == 0u) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        // per digit: exclusive prefix over warps, then advance the base
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < NW; w++) {
            const uint32_t c = wcnt[w][t];
            wcnt[w][t] = run;
            run += c;
        }
        __syncthreads();
        if (valid) {
            const uint32_t dst = base[d] + wcnt[warp][d] + wrank;
            kout[dst] = key;
            vout[dst] = val;
        }
        __syncthreads();
        base[t] += run;
#pragma unroll
        for (int w = 0; w < NW; w++) wcnt[w][t] = 0;
        __syncthreads();
    }
}

static void rs_passes(uint32_t* k0, int* v0, uint32_t* k1, int* v1, uint32_t* hist, uint32_t* tot,
                      int n, int nblocks, int first_pass, int npasses, cudaStream_t st,
                      const Ctl* ctl, int gated) {
    uint32_t* ks[2] = {k0, k1};
    int* vs[2] = {v0, v1};
    for (int p = 0; p < npasses; p++) {
        const int shift = 8 * (first_pass + p);
        const int a = p & 1;
        k_rs_upsweep<<<nblocks, RS_THREADS, 0, st>>>(ks[a], n, shift, hist, nblocks, ctl, gated);
        if (nblocks <= RS_SMALL_TILES) {
            k_rs_downsweep<true><<<nblocks, RS_THREADS, 0, st>>>(ks[a], vs[a], ks[a ^ 1], vs[a ^ 1], n, shift,
                                                                 hist, tot, nblocks, ctl, gated);
        } else {
            k_rs_scan<<<256, 1024, 0, st>>>(hist, nblocks, tot, ctl, gated);
            k_rs_downsweep<false><<<nblocks, RS_THREADS, 0, st>>>(ks[a], vs[a], ks[a ^ 1], vs[a ^ 1], n, shift,
                                                                  hist, tot, nblocks, ctl, gated);
        }
    }
}

void radix_sort_pairs(uint32_t* keys0, int* vals0, uint32_t* keys1, int* vals1, uint32_t* hist,
                      uint32_t* tot, int n, int nblocks, int first_pass, int npasses,
                      cudaStream_t st) {
    rs_passes(keys0, vals0, keys1, vals1, hist, tot, n, nblocks, first_pass, npasses, st, nullptr, 0);
}

// ===================================================================== keys
// Morton key of every particle from its ghost-offset cell coordinates
// (update_pList_withSort, BoundingBox.cu:680-690).  Inactive particles get an
// all-ones key so they sort behind every cell; a particle leaving the box this
// step (status 2) is still keyed, like the reference CPU loop still lists it.
template <class T>
__global__ void k_keys(View<T> v, int gated) {
    const Ctl* ctl = v.ctl;
    if (gated && ctl->refresh == 0u) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.n) return;
    const SBank<T> S = v.S[ctl->s];
    uint32_t key = kNoKey;
    if (S.rot[i].w != 0) {
        const double4_32a p = load_pos(S, i);
        const int cx = cell_x(v, p.x);
        const int cy = cell_coord(p.y, v.miny, v.invdy);
        const int cz = cell_coord(p.z, v.minz, v.invdz);
        key = morton3((uint32_t)cx, (uint32_t)cy, (uint32_t)cz);
    }
    v.keys[0][i] = key;
    v.vals[0][i] = i;
}

// Deactivate particles that left the box at the last step (status 2 -> 0);
// runs before a rebuild requested between steps.
template <class T>
__global__ void k_finalize_oob(View<T> v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.n) return;
    const SBank<T> S = v.S[v.ctl->s];
    if (S.rot[i].w == 2) S.rot[i].w = 0;  // (mixed: posh.w is already negative)
}

template <class T>
void launch_finalize_oob(const View<T>& v, cudaStream_t st) {
    k_finalize_oob<T><<<(v.n + kBlock - 1) / kBlock, kBlock, 0, st>>>(v);
}

// ===================================================================== reorder
// Mixed mode: the inverse of the sort permutation, for remapping the history
// keys (storage indices of contact partners) when the particles move.
template <class T>
__global__ void k_inverse_order(View<T> v, int gated) {
    const Ctl* ctl = v.ctl;
    if (gated && ctl->refresh == 0u) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.n) return;
    v.inv[v.vals[0][i]] = i;
}

// Gather every per-particle array into sorted order (d_swap_ps,
// BoundingBox.cu:928-1005, but with compact histories: only live slots move).
template <class T>
__global__ void __launch_bounds__(kBlock, 4) k_reorder(View<T> v, int gated) {
    Ctl* ctl = v.ctl;
    if (gated && ctl->refresh == 0u) return;
    const int s = ctl->s, p = ctl->p;
    const int n = v.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const int src = v.vals[0][i];
        const SBank<T> A = v.S[s], B = v.S[s ^ 1];
        if (!T::mixed) B.pos[i] = A.pos[src];
        B.vel[i] = A.vel[src];
        B.rot[i] = A.rot[src];
        if (T::mixed) {
            B.posh[i] = A.posh[src];
            B.posl[i] = A.posl[src];
            B.vell[i] = A.vell[src];
            B.rotl[i] = A.rotl[src];
        }
        const PBank<T> P = v.P[p], Q = v.P[p ^ 1];
        Q.mat[i] = P.mat[src];
        Q.pid[i] = P.pid[src];
        // live history slots, four at a time with their loads in flight
        // together (the slot rows are slot-major: slot k of particle i at
        // k * n + i, so a warp's loads of one slot are contiguous)
        using R = typename T::real;
        const int nc = P.nc[src];
        Q.nc[i] = nc;
        for (int k0 = 0; k0 < nc; k0 += 4) {
            int id[4];
            R t[6][4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (k0 + q >= nc) continue;
                const size_t a = (size_t)(k0 + q) * n + src;
                id[q] = P.hid[a];
                t[0][q] = P.hx[a]; t[1][q] = P.hy[a]; t[2][q] = P.hz[a];
                if (T::mixed) { t[3][q] = P.cx[a]; t[4][q] = P.cy[a]; t[5][q] = P.cz[a]; }
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (k0 + q >= nc) continue;
                const size_t b = (size_t)(k0 + q) * n + i;
                Q.hid[b] = T::mixed ? v.inv[id[q]] : id[q];
                Q.hx[b] = t[0][q]; Q.hy[b] = t[1][q]; Q.hz[b] = t[2][q];
                if (T::mixed) { Q.cx[b] = t[3][q]; Q.cy[b] = t[4][q]; Q.cz[b] = t[5][q]; }
            }
        }
        const int ncw = P.ncw[src];
        Q.ncw[i] = ncw;
        for (int k0 = 0; k0 < ncw; k0 += 2) {
            int id[2];
            R t[6][2];
#pragma unroll
            for (int q = 0; q < 2; q++) {
                if (k0 + q >= ncw) continue;
                const size_t a = (size_t)(k0 + q) * n + src;
                id[q] = P.hwid[a];
                t[0][q] = P.hwx[a]; t[1][q] = P.hwy[a]; t[2][q] = P.hwz[a];
                if (T::mixed) { t[3][q] = P.cwx[a]; t[4][q] = P.cwy[a]; t[5][q] = P.cwz[a]; }
            }
#pragma unroll
            for (int q = 0; q < 2; q++) {
                if (k0 + q >= ncw) continue;
                const size_t b = (size_t)(k0 + q) * n + i;
                Q.hwid[b] = id[q];
                Q.hwx[b] = t[0][q]; Q.hwy[b] = t[1][q]; Q.hwz[b] = t[2][q];
                if (T::mixed) { Q.cwx[b] = t[3][q]; Q.cwy[b] = t[4][q]; Q.cwz[b] = t[5][q]; }
            }
        }
    }
    if (last_block(&ctl->done[1])) {
        if (threadIdx.x == 0) {
            ctl->done[1] = 0;
            ctl->s = s ^ 1;
            ctl->p = p ^ 1;
        }
    }
}

// Per-step force/torque outputs follow the particles they belong to.
template <class T>
__global__ void k_reorder_forces(View<T> v, int gated) {
    const Ctl* ctl = v.ctl;
    if (gated && ctl->refresh == 0u) return;
    const int n = v.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int src = v.vals[0][i];
    double* f[6] = {v.fx, v.fy, v.fz, v.tx, v.ty, v.tz};
    for (int c = 0; c < 6; c++) v.ftmp[(size_t)c * n + i] = f[c][src];
}
template <class T>
__global__ void k_copy_forces(View<T> v, int gated) {
    const Ctl* ctl = v.ctl;
    if (gated && ctl->refresh == 0u) return;
    const int n = v.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double* f[6] = {v.fx, v.fy, v.fz, v.tx, v.ty, v.tz};
    for (int c = 0; c < 6; c++) f[c][i] = v.ftmp[(size_t)c * n + i];
}

// ===================================================================== cells
template <class T>
__global__ void k_cells_clear(View<T> v, int gated) {
    const Ctl* ctl = v.ctl;
    if (gated && ctl->refresh == 0u) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) v.ctl->wall_alloc = 0u;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < v.ncells; c += gridDim.x * blockDim.x) {
        v.cell_start[c] = 0;
        v.cell_end[c] = 0;
    }
}

// Cell ranges from the sorted keys: equal keys are one cell, found by
// comparing neighbours in the sorted order (no atomics; replaces
// dk_build_cellCount + ExclusiveSum + dk_build_pList, BoundingBox.cu:1266).
template <class T>
__global__ void k_cell_ranges(View<T> v, int gated) {
    const Ctl* ctl = v.ctl;
    if (gated && ctl->refresh == 0u) return;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = v.n;
    if (q >= n) return;
    // storage index of every pId (the Verlet rows are built as pIds)
    const int jq = v.reorder ? q : v.vals[0][q];
    v.where[v.P[ctl->p].pid[jq]] = jq;
    const uint32_t* key = v.keys[0];
    const uint32_t kq = key[q];
    if (kq == kNoKey) {
        v.nnei[jq] = 0;  // in no cell: an empty Verlet row
        return;
    }
    const int cx = (int)compact10(kq >> 2), cy = (int)compact10(kq >> 1), cz = (int)compact10(kq);
    if (cx >= v.sizex || cy >= v.sizey || cz >= v.sizez) {
        atomicOr(&v.ctl->error, 0x40u);
        v.nnei[jq] = 0;
        return;
    }
    const int cell = (v.sizey * cz + cy) * v.sizex + cx;
    if (q == 0 || key[q - 1] != kq) v.cell_start[cell] = q;
    if (q == n - 1 || key[q + 1] != kq) v.cell_end[cell] = q + 1;
}

// The occupied cells in sorted (Morton) order: the first sorted position of
// every cell inside the grid, compacted by a count per block of kBlock
// positions, one exclusive scan over the blocks and an emit that ranks each
// start within its block.  Neighbouring entries are neighbouring cells, so
// the wall-candidate traversals of neighbouring threads (k_cell_walls) walk
// much the same part of the mesh tree.
template <class T>
__device__ __forceinline__ bool is_cell_start(const View<T>& v, int q) {
    if (q >= v.n) return false;
    const uint32_t* key = v.keys[0];
    const uint32_t kq = key[q];
    if (kq == kNoKey || (q > 0 && key[q - 1] == kq)) return false;
    return (int)compact10(kq >> 2) < v.sizex && (int)compact10(kq >> 1) < v.sizey && (int)compact10(kq) < v.sizez;
}

template <class T>
__global__ void __launch_bounds__(kBlock) k_cell_count(View<T> v, int gated) {
    if (gated && v.ctl->refresh == 0u) return;
    const int c = __syncthreads_count(is_cell_start(v, blockIdx.x * blockDim.x + threadIdx.x));
    if (threadIdx.x == 0) v.cell_bc[blockIdx.x] = c;
}

// Exclusive scan of the nb block counts in place, by one CTA of 1024 threads
// (each a run of consecutive counts); the total goes to ctl->ncell_list.
template <class T>
__global__ void __launch_bounds__(1024) k_cell_scan(View<T> v, int gated, int nb) {
    if (gated && v.ctl->refresh == 0u) return;
    __shared__ int part[1024];
    const int t = threadIdx.x;
    const int per = (nb + 1023) / 1024;
    const int lo = t * per, hi = min(lo + per, nb);
    int sum = 0;
    for (int b = lo; b < hi; b++) sum += v.cell_bc[b];
    part[t] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int add = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += add;
        __syncthreads();
    }
    int run = part[t] - sum;  // exclusive prefix of this run
    for (int b = lo; b < hi; b++) {
        const int c = v.cell_bc[b];
        v.cell_bc[b] = run;
        run += c;
    }
    if (t == 1023) v.ctl->ncell_list = (unsigned)part[1023];
}

template <class T>
__global__ void __launch_bounds__(kBlock) k_cell_emit(View<T> v, int gated) {
    if (gated && v.ctl->refresh == 0u) return;
    __shared__ int wbase[kBlock / 32];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const bool f = is_cell_start(v, q);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned m = __ballot_sync(0xffffffffu, f);
    if (lane == 0) wbase[w] = __popc(m);
    __syncthreads();
    if (f) {
        int off = v.cell_bc[blockIdx.x];
        for (int u = 0; u < w; u++) off += wbase[u];
        v.cell_list[off + __popc(m & ((1u << lane) - 1u))] = q;
    }
}

// ===================================================================== Verlet lists
// FP64 mode: FP32 copy of the positions for the prefilter of k_neighbors.
template <class T>
__global__ void k_posf(View<T> v, int gated) {
    const Ctl* ctl = v.ctl;
    if (gated && ctl->refresh == 0u) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.n) return;
    const double4_32a p = v.S[ctl->s].pos[i];
    v.posf[i] = make_float4((float)p.x, (float)p.y, (float)p.z, (float)p.w);
}

// One thread per particle: scan the 27 cells around its cell, keep every
// listed j != i with |xi - xj|^2 < (ri + rj + skin)^2 (the test of
// BoundingBox.cu:1136-1144, FP64 in every mode), order the row by the
// partner's pId (the reference's index space) and record the reference
// position.  Cells outside the grid hold nobody and are skipped.
//
// Most candidates are far from the cutoff, so each is first tested on FP32
// positions: nb_delta bounds how far the FP32 distance can be from the FP64
// one (eight FP32 ulps of the largest box coordinate, more than the two
// roundings of the coordinates), and only a candidate whose FP32 distance is
// within that band of the cutoff takes the FP64 test.  The decision is the
// FP64 test's in every case.
//
// The row grows in shared memory as partner pIds (slot k of thread t at
// k * kNbBlock + t: the threads of a warp touch 32 banks), is sorted by
// insertion once the scan is done, and is written out once, mapped back to
// storage indices through v.where, slot by slot (a warp writes 32
// consecutive ints per slot).
constexpr int kNbBlock = 128;
constexpr int kNbUnroll = 4;

template <int CAP>
constexpr size_t nb_smem_bytes() {
    return sizeof(int) * (size_t)CAP * kNbBlock;
}

template <class T, int CAP>
__global__ void __launch_bounds__(kNbBlock) k_neighbors(View<T> v, int gated) {
    extern __shared__ int nb_rows[];
    Ctl* ctl = v.ctl;
    if (gated && ctl->refresh == 0u) return;
    const int n = v.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = ctl->s, p = ctl->p;
    const SBank<T> S = v.S[s];
    const PBank<T> P = v.P[p];
    const float4* __restrict__ PF = T::mixed ? S.posh : v.posf;
    const int* __restrict__ pidv = P.pid;
    int* row = nb_rows + threadIdx.x;
    int count = 0;
    if (i < n) {
        if (S.rot[i].w == 0) {
            v.nnei[i] = 0;
        } else {
            const double4_32a pi = load_pos(S, i);
            const float4 fi = PF[i];
            const double xi = pi.x, yi = pi.y, zi = pi.z, ri = pi.w;
            const double skin = v.skin;
            const float skinf = (float)v.skin, delta = v.nb_delta;
            const float rfi = fabsf(fi.w) + skinf;
            const int cx = cell_x(v, xi);
            const int cy = cell_coord(yi, v.miny, v.invdy);
            const int cz = cell_coord(zi, v.minz, v.invdz);
            bool overflow = false;
            for (int sz = -1; sz <= 1; sz++) {
                const int zz = cz + sz;
                if (zz < 0 || zz >= v.sizez) continue;
                for (int sy = -1; sy <= 1; sy++) {
                    const int yy = cy + sy;
                    if (yy < 0 || yy >= v.sizey) continue;
                    for (int sx = -1; sx <= 1; sx++) {
                        int xx = cx + sx;
                        if (v.per_x) {
                            // cells 1..nxp wrap around (nxp >= 3: no cell twice)
                            if (xx < 1) xx += v.nxp;
                            else if (xx > v.nxp) xx -= v.nxp;
                        } else if (xx < 0 || xx >= v.sizex) {
                            continue;
                        }
                        const int cell = (v.sizey * zz + yy) * v.sizex + xx;
                        const int b = v.cell_start[cell], e = v.cell_end[cell];
                        // kNbUnroll candidates at a time, their loads in flight together
                        for (int q0 = b; q0 < e; q0 += kNbUnroll) {
                            int jj[kNbUnroll];
                            float4 fj[kNbUnroll];
#pragma unroll
                            for (int u = 0; u < kNbUnroll; u++) {
                                const int q = q0 + u;
                                jj[u] = q < e ? (v.reorder ? q : v.vals[0][q]) : -1;
                                if (jj[u] >= 0) fj[u] = PF[jj[u]];
                            }
#pragma unroll
                            for (int u = 0; u < kNbUnroll; u++) {
                                const int j = jj[u];
                                if (j < 0 || j == i) continue;
                                const float ex = image_dxf(v, fi.x - fj[u].x), ey = fi.y - fj[u].y,
                                            ez = fi.z - fj[u].z;
                                const float dsqf = ex * ex + ey * ey + ez * ez;
                                const float Rf = rfi + fabsf(fj[u].w);
                                const float Rhi = Rf + delta;
                                if (dsqf > Rhi * Rhi * 1.0000039f) continue;  // (1 + 2^-18): surely outside
                                const float Rlo = Rf - delta;
                                bool inside = Rlo > 0.f && dsqf < Rlo * Rlo * 0.9999962f;  // surely inside
                                if (!inside) {
                                    const double4_32a pj = load_pos(S, j);
                                    const double dx = image_dx(v, xi - pj.x);
                                    const double dy = yi - pj.y;
                                    const double dz = zi - pj.z;
                                    const double distsq = dx * dx + dy * dy + dz * dz;
                                    const double R = ri + pj.w + skin;
                                    inside = distsq < R * R;
                                }
                                if (!inside) continue;
                                if (count >= CAP) {
                                    overflow = true;
                                    continue;
                                }
                                row[count * kNbBlock] = pidv[j];  // sorted once the scan is done
                                count++;
                            }
                        }
                    }
                }
            }
            if (overflow || count > v.nei_cap) atomicOr(&ctl->error, 0x1u);
            // the row by pId: an insertion sort after the scan, run by all the
            // warp's lanes together rather than one lane per hit during it
            const int cs = count < CAP ? count : CAP;
            for (int a = 1; a < cs; a++) {
                const int key = row[a * kNbBlock];
                int b = a;
                while (b > 0) {
                    const int prev = row[(b - 1) * kNbBlock];
                    if (prev < key) break;
                    row[b * kNbBlock] = prev;
                    b--;
                }
                row[b * kNbBlock] = key;
            }
            const int m = count < v.nei_cap ? count : v.nei_cap;
            for (int k = 0; k < m; k++) v.nei[(size_t)k * n + i] = v.where[row[k * kNbBlock]];
            v.nnei[i] = m;
            if (T::mixed)
                v.refh[i] = make_float4(fi.x, fi.y, fi.z, 0.f);
            else
                v.ref[i] = make_double4_32a(xi, yi, zi, 0.0);
        }
    }
    int wmax = count;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
    if ((threadIdx.x & 31) == 0 && wmax > 0) atomicMax(&ctl->max_nei, wmax);
}

template <class T, int CAP>
static void launch_neighbors(const View<T>& v, int gated, cudaStream_t st) {
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(k_neighbors<T, CAP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)nb_smem_bytes<CAP>());
        configured = true;
    }
    k_neighbors<T, CAP><<<(v.n + kNbBlock - 1) / kNbBlock, kNbBlock, nb_smem_bytes<CAP>(), st>>>(v, gated);
}

// ===================================================================== wall lists
// Mesh tree traversal with an explicit stack; a triangle joins the list when
// its AABB and its closest feature are within r + skin (BVH.cu:493-540, with
// sphereAABBOverlapNeighbor and dist_triangle_neighbor).  The set does not
// depend on the tree shape: an ancestor's box contains its leaves' boxes, so
// the box test never rejects an ancestor of a leaf that passes.  Rows are
// sorted by triangle index, as BVH.cu:538 does.

// children of mesh tree node (L, k), L > 0, pushed right first
__device__ __forceinline__ bool seg_push(unsigned* stack, int& sp, int L, int k, int ntri) {
    if (sp + 2 > kBvhStack) return false;
    const int below = (ntri + (1 << (L - 1)) - 1) >> (L - 1);
    const unsigned lv = (unsigned)(L - 1) << kSegShift;
    if (2 * k + 1 < below) stack[sp++] = lv | (unsigned)(2 * k + 1);
    stack[sp++] = lv | (unsigned)(2 * k);
    return true;
}
// Wall candidates of every occupied cell, one thread per listed cell: the
// mesh tree's FP32 boxes (rounded outwards) traversed with the cell's box
// grown by v.cw_reach (every particle's cutoff r + skin, the mixed rows'
// widening, a margin) and rounded outwards too, every triangle whose box
// overlaps it, ascending.  An ancestor's box contains its leaves', and every
// rounding widens a box, so no leaf that a particle's own tree test (sphere
// against the triangle's box) would pass is left out.  A periodic x also
// takes the cell's box one period away where it reaches over an x face.  A
// cell with more than kCellWalls candidates, or one that finds the buffer
// full, is marked -1 and its particles traverse the tree themselves.
constexpr int kCellWalls = 96;

template <class T>
__global__ void __launch_bounds__(kBlock) k_cell_walls(View<T> v, int gated) {
    Ctl* ctl = v.ctl;
    if (gated && ctl->refresh == 0u) return;
    const int c_idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (c_idx >= (int)ctl->ncell_list) return;
    const int q = v.cell_list[c_idx];
    const uint32_t kq = v.keys[0][q];
    const int c[3] = {(int)compact10(kq >> 2), (int)compact10(kq >> 1), (int)compact10(kq)};
    if (v.ntri == 0) {
        v.cw_cnt[q] = 0;
        return;
    }
    const double reach = v.cw_reach + (T::mixed ? (double)v.wall_delta : 0.);
    const double mn[3] = {v.minx, v.miny, v.minz};
    const double inv[3] = {v.invdx, v.invdy, v.invdz};
    double lo[3], hi[3];
    for (int a = 0; a < 3; a++) {
        lo[a] = mn[a] + (double)(c[a] - 1) / inv[a] - reach;
        hi[a] = mn[a] + (double)c[a] / inv[a] + reach;
    }
    const int nimg = v.per_x && (hi[0] > v.maxx || lo[0] < v.minx) ? 2 : 1;
    int cand[kCellWalls];
    int count = 0;
    bool full = false;
    unsigned stack[kBvhStack];
    for (int img = 0; img < nimg && !full; img++) {
        const double shift = img == 0 ? 0. : (hi[0] > v.maxx ? -v.Lx : v.Lx);
        // the grown box in FP32, rounded outwards
        float flo[3], fhi[3];
        for (int a = 0; a < 3; a++) {
            const double l = lo[a] + (a == 0 ? shift : 0.), h = hi[a] + (a == 0 ? shift : 0.);
            flo[a] = __double2float_rd(l);
            fhi[a] = __double2float_ru(h);
        }
        int sp = 0;
        stack[sp++] = (unsigned)v.seg_top << kSegShift;
        while (sp > 0) {
            const unsigned e = stack[--sp];
            const int L = (int)(e >> kSegShift), nk = (int)(e & ((1u << kSegShift) - 1u));
            const SegBoxF B = v.segf[v.seg_off[L] + nk];
            if (B.lo[0] > fhi[0] || B.hi[0] < flo[0] || B.lo[1] > fhi[1] || B.hi[1] < flo[1] || B.lo[2] > fhi[2] ||
                B.hi[2] < flo[2])
                continue;
            if (L == 0) {
                const int t = v.seg_tri[nk];
                if (count >= kCellWalls) {
                    full = true;
                    break;
                }
                int k = count;
                while (k > 0 && cand[k - 1] > t) {
                    cand[k] = cand[k - 1];
                    k--;
                }
                if (k > 0 && cand[k - 1] == t) {  // met at the other image already
                    for (int u = k; u < count; u++) cand[u] = cand[u + 1];
                    continue;
                }
                cand[k] = t;
                count++;
            } else if (!seg_push(stack, sp, L, nk, v.ntri)) {
                full = true;
                break;
            }
        }
    }
    int base = 0;
    if (!full && count > 0) {
        base = (int)atomicAdd(&ctl->wall_alloc, (unsigned)count);
        if (base + count > v.cw_cap) full = true;
    }
    if (full) {
        v.cw_cnt[q] = -1;
        return;
    }
    for (int k = 0; k < count; k++) v.cw_list[base + k] = cand[k];
    v.cw_base[q] = base;
    v.cw_cnt[q] = count;
}

// The cell wall candidates of particle i's cell (first sorted position q0 and
// count), or count -1 when its particles traverse the tree themselves.
template <class T>
__device__ __forceinline__ int cell_walls_of(const View<T>& v, double x, double y, double z, int& base) {
    const int cx = cell_x(v, x), cy = cell_coord(y, v.miny, v.invdy), cz = cell_coord(z, v.minz, v.invdz);
    if (cx < 0 || cx >= v.sizex || cy < 0 || cy >= v.sizey || cz < 0 || cz >= v.sizez) return -1;
    const int cell = (v.sizey * cz + cy) * v.sizex + cx;
    if (v.cell_end[cell] <= v.cell_start[cell]) return -1;
    const int q0 = v.cell_start[cell];
    base = v.cw_base[q0];
    return v.cw_cnt[q0];
}

template <class T, int CAP>
__global__ void __launch_bounds__(kBlock) k_wall_lists(View<T> v, int gated) {
    Ctl* ctl = v.ctl;
    if (gated && ctl->refresh == 0u) return;
    const int n = v.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = ctl->s;
    int count = 0;
    if (i < n) {
        const SBank<T> S = v.S[s];
        if (S.rot[i].w == 0 || v.ntri == 0) {
            v.nneiw[i] = 0;
        } else if constexpr (T::mixed) {
            // FP32 traversal of the FP32 tree (boxes rounded outwards) and the
            // FP32 closest feature, with the cutoff widened by their error
            // bounds: the rows hold every triangle within r + skin (and maybe
            // a few more, which the step's exact overlap turns away), so the
            // contacts are those of the FP64 rows
            const float4 h = S.posh[i], l = S.posl[i];
            const float3 pl = make_float3(l.x, l.y, l.z);
            const float R = fabsf(h.w) + l.w + (float)v.skin + v.nb_delta + v.wall_delta;
            const float Rsq = R * R;
            int cand[CAP];
            bool overflow = false;
            int cbase = 0;
            const int ccnt = cell_walls_of(v, (double)h.x + (double)l.x, (double)h.y + (double)l.y,
                                           (double)h.z + (double)l.z, cbase);
            if (ccnt >= 0) {
                // the cell's candidates, ascending: the row comes out sorted
                for (int k = 0; k < ccnt; k++) {
                    const int t = v.cw_list[cbase + k];
                    float3 qh = make_float3(h.x, h.y, h.z), ql = pl;
                    if (v.per_x) {
                        const float d = qh.x - v.trif[t].v0h[0];
                        if (d > v.halfLxf || d < -v.halfLxf) {
                            qh.x = d > 0.f ? qh.x - v.Lxh : qh.x + v.Lxh;
                            ql.x = 0.f;  // the period's low part is within the margin
                        }
                    }
                    const FeatureF f = closest_feature_f(qh, ql, Rsq, v.trif[t]);
                    if (!(f.dist < R)) continue;
                    if (count >= CAP) {
                        overflow = true;
                        break;
                    }
                    cand[count++] = t;
                }
            }
            unsigned stack[kBvhStack];
            const int nimg = ccnt >= 0 ? 0 : (v.per_x && (h.x + R > v.perf[1] || h.x - R < v.perf[0]) ? 2 : 1);
            for (int img = 0; img < nimg; img++) {
                float3 ph = make_float3(h.x, h.y, h.z);
                if (img == 1) ph.x = h.x + R > v.perf[1] ? h.x - v.Lxh : h.x + v.Lxh;
                int sp = 0;
                stack[sp++] = (unsigned)v.seg_top << kSegShift;
                while (sp > 0) {
                    const unsigned e = stack[--sp];
                    const int L = (int)(e >> kSegShift), nk = (int)(e & ((1u << kSegShift) - 1u));
                    const SegBoxF N = v.segf[v.seg_off[L] + nk];
                    const float dx = fmaxf(fmaxf(N.lo[0] - ph.x, ph.x - N.hi[0]), 0.f);
                    const float dy = fmaxf(fmaxf(N.lo[1] - ph.y, ph.y - N.hi[1]), 0.f);
                    const float dz = fmaxf(fmaxf(N.lo[2] - ph.z, ph.z - N.hi[2]), 0.f);
                    if (!(dx * dx + dy * dy + dz * dz <= Rsq)) continue;
                    if (L == 0) {
                        const int t = v.seg_tri[nk];
                        float3 qh = ph, ql = pl;
                        if (img == 1) ql.x = 0.f;  // the period's low part is within the margin
                        const FeatureF f = closest_feature_f(qh, ql, Rsq, v.trif[t]);
                        if (f.dist < R) {
                            if (count >= CAP) {
                                overflow = true;
                                continue;
                            }
                            int k = count;
                            while (k > 0 && cand[k - 1] > t) {
                                cand[k] = cand[k - 1];
                                k--;
                            }
                            cand[k] = t;
                            count++;
                        }
                    } else if (!seg_push(stack, sp, L, nk, v.ntri)) {
                        atomicOr(&ctl->error, 0x10u);
                        break;
                    }
                }
            }
            if (overflow || count > v.wall_cap) atomicOr(&ctl->error, 0x2u);
            const int m = count < v.wall_cap ? count : v.wall_cap;
            for (int k = 0; k < m; k++) v.neiw[(size_t)k * n + i] = cand[k];
            v.nneiw[i] = m;
        } else {
            const double4_32a pi = load_pos(S, i);
            const double py = pi.y, pz = pi.z;
            const double R = pi.w + v.skin;
            const double Rsq = R * R;
            int cand[CAP];
            bool overflow = false;
            int cbase = 0;
            const int ccnt = cell_walls_of(v, pi.x, py, pz, cbase);
            if (ccnt >= 0) {
                // the cell's candidates, ascending, through the same two tests
                // as the traversal below (sphere against the triangle's box,
                // then the closest feature): the same row, already sorted
                for (int k = 0; k < ccnt; k++) {
                    const int t = v.cw_list[cbase + k];
                    const double px = image_x_near(v, pi.x, v.tri[t].v0[0]);
                    const double* bb = v.tri_aabb + 6 * (size_t)t;
                    if (!sphere_aabb(px, py, pz, Rsq, bb, bb + 3)) continue;
                    const Feature f = closest_feature(px, py, pz, Rsq, v.tri[t]);
                    if (!(f.dist < pi.w + v.skin)) continue;
                    if (count >= CAP) {
                        overflow = true;
                        break;
                    }
                    cand[count++] = t;
                }
            }
            unsigned stack[kBvhStack];
            // periodic x: a sphere within R of an x face also queries the mesh
            // at its image one period away (no triangle is found twice: the
            // mesh's triangles are narrower than a quarter period)
            const int nimg = ccnt >= 0 ? 0 : (v.per_x && (pi.x + R > v.maxx || pi.x - R < v.minx) ? 2 : 1);
            for (int img = 0; img < nimg; img++) {
                const double px = img == 0 ? pi.x : (pi.x + R > v.maxx ? pi.x - v.Lx : pi.x + v.Lx);
                int sp = 0;
                stack[sp++] = (unsigned)v.seg_top << kSegShift;
                while (sp > 0) {
                    const unsigned e = stack[--sp];
                    const int L = (int)(e >> kSegShift), nk = (int)(e & ((1u << kSegShift) - 1u));
                    const SegBox& B = v.seg[v.seg_off[L] + nk];
                    if (!sphere_aabb(px, py, pz, Rsq, B.lo, B.hi)) continue;
                    if (L == 0) {
                        const int t = v.seg_tri[nk];
                        const Feature f = closest_feature(px, py, pz, Rsq, v.tri[t]);
                        if (f.dist < pi.w + v.skin) {
                            if (count >= CAP) {
                                overflow = true;
                                continue;
                            }
                            int k = count;
                            while (k > 0 && cand[k - 1] > t) {
                                cand[k] = cand[k - 1];
                                k--;
                            }
                            cand[k] = t;
                            count++;
                        }
                    } else if (!seg_push(stack, sp, L, nk, v.ntri)) {
                        atomicOr(&ctl->error, 0x10u);
                        break;
                    }
                }
            }
            if (overflow || count > v.wall_cap) atomicOr(&ctl->error, 0x2u);
            const int m = count < v.wall_cap ? count : v.wall_cap;
            for (int k = 0; k < m; k++) v.neiw[(size_t)k * n + i] = cand[k];
            v.nneiw[i] = m;
        }
    }
    int wmax = count;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
    if ((threadIdx.x & 31) == 0 && wmax > 0) atomicMax(&ctl->max_wall, wmax);
    // the last block closes the rebuild: clear the request, count it
    if (last_block(&ctl->done[2])) {
        if (threadIdx.x == 0) {
            ctl->done[2] = 0;
            ctl->refresh = 0u;
            ctl->rebuilds += 1ull;
            ctl->lists_valid = 1;
            ctl->irefresh = 1u;  // new list rows (and storage order): new inner rows
        }
    }
}

// ===================================================================== inner rows
// Mixed mode: the partners of each list row within r_i + r_j + inner skin,
// in row order (so in partner-pId order), the wall-row triangles within
// r_i + inner skin (FP64 closest feature, in row order), and the high-part
// positions they were taken at.  The test runs on the high parts with the list prefilter's
// error bound added to the cutoff, so it keeps every pair that is within the
// cutoff in exact arithmetic.  A pair left out is more than the inner skin
// apart, and it cannot touch before some particle has moved half the inner
// skin, when the step asks for new rows (ctl->irefresh); every list rebuild
// asks too.  Gated on that request in every launch mode.
constexpr int kInnerKeys = 8;
// row entries in flight per thread: 4 measured 180 us on the 1M bed, 8 and 16
// (more registers, fewer resident warps) 207 and 277 us
constexpr int kInnerUnroll = 4;

template <class T>
__global__ void __launch_bounds__(kBlock) k_inner(View<T> v) {
    Ctl* ctl = v.ctl;
    if (ctl->irefresh == 0u) return;
    const int n = v.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (T::mixed) {
        if (i < n) {
            const SBank<T> S = v.S[ctl->s];
            const float4 hi = S.posh[i];
            int m = 0;
            if (hi.w > 0.f) {
                const int nn = v.nnei[i];
                const float cut = v.inner_skinf + v.nb_delta;
                const bool hints = v.row_mask != 0xFFFFFFFFu;
                const PBank<T> P = v.P[ctl->p];
                // the first kInnerKeys history keys in registers for the
                // slot hints (the rest, rarely used, read when needed)
                const int nc = hints ? P.nc[i] : 0;
                int hk[kInnerKeys];
#pragma unroll
                for (int q = 0; q < kInnerKeys; q++) hk[q] = q < nc ? P.hid[(size_t)q * n + i] : -1;
                // kInnerUnroll row entries at a time, their gathers in flight together
                for (int k0 = 0; k0 < nn; k0 += kInnerUnroll) {
                    int jj[kInnerUnroll];
                    float4 hj[kInnerUnroll];
#pragma unroll
                    for (int u = 0; u < kInnerUnroll; u++) jj[u] = k0 + u < nn ? v.nei[(size_t)(k0 + u) * n + i] : -1;
#pragma unroll
                    for (int u = 0; u < kInnerUnroll; u++)
                        if (jj[u] >= 0) hj[u] = S.posh[jj[u]];
#pragma unroll
                    for (int u = 0; u < kInnerUnroll; u++) {
                        const int j = jj[u];
                        if (j < 0 || !(hj[u].w > 0.f)) continue;  // inactive for good
                        const float dx = image_dxf(v, hi.x - hj[u].x), dy = hi.y - hj[u].y, dz = hi.z - hj[u].z;
                        const float R = hi.w + hj[u].w + cut;
                        if (!(dx * dx + dy * dy + dz * dz < R * R * 1.0000039f)) continue;
                        if (m < v.nei_cap) {
                            // the partner's history slot, if it has one, as a hint
                            int e = j;
                            if (hints) {
                                int q = -1;
#pragma unroll
                                for (int a = 0; a < kInnerKeys; a++)
                                    if (q < 0 && hk[a] == j) q = a;
                                for (int a = kInnerKeys; q < 0 && a < nc && a < 63; a++)
                                    if (P.hid[(size_t)a * n + i] == j) q = a;
                                if (q >= 0) e = j | ((q + 1) << kHintShift);
                            }
                            v.inn[(size_t)m * n + i] = e;
                        }
                        m++;
                    }
                }
            }
            v.ninn[i] = m < v.nei_cap ? m : v.nei_cap;
            int mw = 0;
            if (hi.w > 0.f && v.ntri > 0) {
                // FP32 closest feature with the cutoff widened by its error bound
                const float4 lo = S.posl[i];
                const float R = hi.w + lo.w + v.inner_skinf + v.nb_delta + v.wall_delta;
                const int nw = v.nneiw[i];
                for (int k = 0; k < nw; k++) {
                    const int t = v.neiw[(size_t)k * n + i];
                    float3 ph = make_float3(hi.x, hi.y, hi.z), pl = make_float3(lo.x, lo.y, lo.z);
                    if (v.per_x) {
                        const float d = ph.x - v.trif[t].v0h[0];
                        if (d > v.halfLxf || d < -v.halfLxf) {
                            ph.x = d > 0.f ? ph.x - v.Lxh : ph.x + v.Lxh;
                            pl.x = 0.f;  // within the margin
                        }
                    }
                    const FeatureF f = closest_feature_f(ph, pl, R * R, v.trif[t]);
                    if (f.dist < R) v.innw[(size_t)mw++ * n + i] = t;
                }
            }
            v.ninnw[i] = mw;
            v.refi[i] = make_float4(hi.x, hi.y, hi.z, 0.f);
        }
    }
    if (last_block(&ctl->done[3])) {
        if (threadIdx.x == 0) {
            ctl->done[3] = 0;
            ctl->irefresh = 0u;
            ctl->inner_builds += 1ull;
        }
    }
}

static inline int grid_for(int n) { return (n + kBlock - 1) / kBlock; }

template <class T>
void launch_inner(const View<T>& v, cudaStream_t st) {
    if (T::mixed && v.inner_on) k_inner<T><<<grid_for(v.n), kBlock, 0, st>>>(v);
}
template void launch_inner<FP64>(const View<FP64>&, cudaStream_t);
template void launch_inner<Mixed>(const View<Mixed>&, cudaStream_t);

template <class T>
void launch_rebuild(const View<T>& v, cudaStream_t st, int force) {
    const int gated = force ? 0 : 1;
    const int n = v.n;
    const int g = grid_for(n);
    k_keys<T><<<g, kBlock, 0, st>>>(v, gated);
    rs_passes(v.keys[0], v.vals[0], v.keys[1], v.vals[1], v.rs_hist, v.rs_tot, n, v.rs_blocks, 0, 4, st,
              v.ctl, gated);
    if (v.reorder) {
        if (v.store_forces) {
            k_reorder_forces<T><<<g, kBlock, 0, st>>>(v, gated);
            k_copy_forces<T><<<g, kBlock, 0, st>>>(v, gated);
        }
        if constexpr (T::mixed) k_inverse_order<T><<<g, kBlock, 0, st>>>(v, gated);
        k_reorder<T><<<g, kBlock, 0, st>>>(v, gated);
    }
    const int gc = grid_for(v.ncells) < 4096 ? grid_for(v.ncells) : 4096;
    k_cells_clear<T><<<gc, kBlock, 0, st>>>(v, gated);
    k_cell_ranges<T><<<g, kBlock, 0, st>>>(v, gated);
    k_cell_count<T><<<g, kBlock, 0, st>>>(v, gated);
    k_cell_scan<T><<<1, 1024, 0, st>>>(v, gated, g);
    k_cell_emit<T><<<g, kBlock, 0, st>>>(v, gated);
    if constexpr (!T::mixed) k_posf<T><<<g, kBlock, 0, st>>>(v, gated);
    if (v.nei_cap <= 32)
        launch_neighbors<T, 32>(v, gated, st);
    else if (v.nei_cap <= 64)
        launch_neighbors<T, 64>(v, gated, st);
    else
        launch_neighbors<T, 128>(v, gated, st);
    k_cell_walls<T><<<g, kBlock, 0, st>>>(v, gated);
    if (v.wall_cap <= 16)
        k_wall_lists<T, 16><<<g, kBlock, 0, st>>>(v, gated);
    else if (v.wall_cap <= 32)
        k_wall_lists<T, 32><<<g, kBlock, 0, st>>>(v, gated);
    else
        k_wall_lists<T, 64><<<g, kBlock, 0, st>>>(v, gated);
    launch_inner(v, st);
}

template void launch_rebuild<FP64>(const View<FP64>&, cudaStream_t, int);
template void launch_rebuild<Mixed>(const View<Mixed>&, cudaStream_t, int);
template void launch_finalize_oob<FP64>(const View<FP64>&, cudaStream_t);
template void launch_finalize_oob<Mixed>(const View<Mixed>&, cudaStream_t);

// ===================================================================== mesh
// Per-triangle precompute of load_ascii_stl_double (TriangleMesh.cu:560-630)
// from welded vertices (tv = sorted vertex ids, te = edge ids + nShift) and
// the raw third corner (the plane offset uses it, TriangleMesh.cu:607) or,
// when raw3 is null, the plane offsets the loader already computed (dplane),
// plus the centroid Morton key of mortonKeyGen (TriangleMesh.cu:4-21).
__global__ void k_tri_precompute(TriRec* rec, uint32_t* morton, int* idx, const double* vx,
                                 const double* vy, const double* vz, const int* tv, const int* te,
                                 const double* raw3, const double* dplane, int ntri, double gminx, double gminy,
                                 double gminz, double irx, double iry, double irz) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    const int a = tv[3 * t + 0], b = tv[3 * t + 1], c = tv[3 * t + 2];
    TriRec R;
    R.v0[0] = vx[a]; R.v0[1] = vy[a]; R.v0[2] = vz[a];
    R.v1[0] = vx[b]; R.v1[1] = vy[b]; R.v1[2] = vz[b];
    R.v2[0] = vx[c]; R.v2[1] = vy[c]; R.v2[2] = vz[c];
    for (int k = 0; k < 3; k++) {
        R.e01[k] = R.v1[k] - R.v0[k];
        R.e02[k] = R.v2[k] - R.v0[k];
        R.e12[k] = R.v2[k] - R.v1[k];
    }
    const double d00 = R.e01[0] * R.e01[0] + R.e01[1] * R.e01[1] + R.e01[2] * R.e01[2];
    const double d01 = R.e01[0] * R.e02[0] + R.e01[1] * R.e02[1] + R.e01[2] * R.e02[2];
    const double d11 = R.e02[0] * R.e02[0] + R.e02[1] * R.e02[1] + R.e02[2] * R.e02[2];
    const double d22 = R.e12[0] * R.e12[0] + R.e12[1] * R.e12[1] + R.e12[2] * R.e12[2];
    R.d00 = d00;
    R.d01 = d01;
    R.d11 = d11;
    R.d00inv = 1. / d00;
    R.d11inv = 1. / d11;
    R.d22inv = 1. / d22;
    R.denom = 1. / (d00 * d11 - d01 * d01);
    // n = normalize(e01 x e02)
    double nx = R.e01[1] * R.e02[2] - R.e01[2] * R.e02[1];
    double ny = R.e01[2] * R.e02[0] - R.e01[0] * R.e02[2];
    double nz = R.e01[0] * R.e02[1] - R.e01[1] * R.e02[0];
    const double inv = 1. / sqrt(nx * nx + ny * ny + nz * nz);
    nx = inv * nx;
    ny = inv * ny;
    nz = inv * nz;
    R.n[0] = nx;
    R.n[1] = ny;
    R.n[2] = nz;
    if (raw3) {
        const double x = raw3[3 * t + 0], y = raw3[3 * t + 1], z = raw3[3 * t + 2];
        R.d = -nx * x - ny * y - nz * z;
    } else {
        R.d = dplane[t];
    }
    R.i0 = a;
    R.i1 = b;
    R.i2 = c;
    R.e0 = te[3 * t + 0];
    R.e1 = te[3 * t + 1];
    R.e2 = te[3 * t + 2];
    rec[t] = R;
    const double cx = (R.v0[0] + R.v1[0] + R.v2[0]) / 3.0;
    const double cy = (R.v0[1] + R.v1[1] + R.v2[1]) / 3.0;
    const double cz = (R.v0[2] + R.v1[2] + R.v2[2]) / 3.0;
    const uint32_t ix = (uint32_t)((cx - gminx) * irx);
    const uint32_t iy = (uint32_t)((cy - gminy) * iry);
    const uint32_t iz = (uint32_t)((cz - gminz) * irz);
    morton[t] = morton3(ix, iy, iz);
    idx[t] = t;
}

void launch_tri_precompute(TriRec* rec, uint32_t* morton, int* idx, const double* vx,
                           const double* vy, const double* vz, const int* tv, const int* te,
                           const double* raw3, const double* dplane, int ntri, const double* gmin,
                           const double* invrange, cudaStream_t st) {
    if (ntri <= 0) return;
    k_tri_precompute<<<grid_for(ntri), kBlock, 0, st>>>(rec, morton, idx, vx, vy, vz, tv, te, raw3, dplane,
                                                        ntri, gmin[0], gmin[1], gmin[2], invrange[0],
                                                        invrange[1], invrange[2]);
}

// Centroid keys of the triangles from their records (the key formula of
// k_tri_precompute), for rebuilding the tree of a mesh already set.
__global__ void k_tri_keys(const TriRec* rec, uint32_t* morton, int* idx, int ntri, double gminx, double gminy,
                           double gminz, double irx, double iry, double irz) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    const TriRec& R = rec[t];
    const double cx = (R.v0[0] + R.v1[0] + R.v2[0]) / 3.0;
    const double cy = (R.v0[1] + R.v1[1] + R.v2[1]) / 3.0;
    const double cz = (R.v0[2] + R.v1[2] + R.v2[2]) / 3.0;
    const uint32_t ix = (uint32_t)((cx - gminx) * irx);
    const uint32_t iy = (uint32_t)((cy - gminy) * iry);
    const uint32_t iz = (uint32_t)((cz - gminz) * irz);
    morton[t] = morton3(ix, iy, iz);
    idx[t] = t;
}

void launch_tri_keys(const TriRec* rec, uint32_t* morton, int* idx, int ntri, const double* gmin,
                     const double* invrange, cudaStream_t st) {
    if (ntri <= 0) return;
    k_tri_keys<<<grid_for(ntri), kBlock, 0, st>>>(rec, morton, idx, ntri, gmin[0], gmin[1], gmin[2], invrange[0],
                                                  invrange[1], invrange[2]);
}

// ---- mesh tree: built per 256 sorted triangles in shared memory by one CTA
// each, the levels above by the last CTA to finish (atomic counter, no
// waiting).

__host__ __device__ __forceinline__ int seg_count(int n, int level) {
    return (int)(((long long)n + (1ll << level) - 1) >> level);
}
__host__ __device__ __forceinline__ int seg_offset(int n, int level) {
    int off = 0;
    for (int L = 0; L < level; L++) off += seg_count(n, L);
    return off;
}
int seg_levels(int n) {
    int L = 0;
    while (seg_count(n, L) > 1) L++;
    return L + 1;
}
int seg_count_host(int n, int level) { return seg_count(n, level); }
int seg_offset_host(int n, int level) { return seg_offset(n, level); }

__device__ __forceinline__ SegBox seg_union(const SegBox& a, const SegBox& b) {
    SegBox c;
    for (int k = 0; k < 3; k++) {
        c.lo[k] = a.lo[k] < b.lo[k] ? a.lo[k] : b.lo[k];
        c.hi[k] = a.hi[k] > b.hi[k] ? a.hi[k] : b.hi[k];
    }
    return c;
}

// boxes written by other CTAs: read through L2
__device__ __forceinline__ SegBox seg_load_cg(const SegBox* p) {
    SegBox b;
    for (int k = 0; k < 3; k++) {
        b.lo[k] = __ldcg(&p->lo[k]);
        b.hi[k] = __ldcg(&p->hi[k]);
    }
    return b;
}

constexpr int kSegTile = 256;
constexpr int kSegTileLevels = 9;  // levels 0..8 inside one CTA's 256 leaves

// box and its FP32 copy (rounded outwards)
__device__ __forceinline__ void put_box(SegBox* seg, SegBoxF* segf, int i, const SegBox& b) {
    seg[i] = b;
    SegBoxF f;
    for (int k = 0; k < 3; k++) {
        f.lo[k] = __double2float_rd(b.lo[k]);
        f.hi[k] = __double2float_ru(b.hi[k]);
    }
    segf[i] = f;
}

__global__ void __launch_bounds__(kSegTile) k_mesh_tree(const double* aabb, const int* sorted_idx, SegBox* seg,
                                                         SegBoxF* segf, unsigned* done, int n) {
    __shared__ SegBox sb[kSegTile];
    const int tid = threadIdx.x;
    const int l = blockIdx.x * kSegTile + tid;
    if (l < n) {
        const int t = sorted_idx[l];
        SegBox b;
        for (int k = 0; k < 3; k++) {
            b.lo[k] = aabb[6 * t + k];
            b.hi[k] = aabb[6 * t + 3 + k];
        }
        put_box(seg, segf, l, b);
        sb[tid] = b;
    }
    __syncthreads();
    // levels 1..8 of this CTA's leaves
    for (int L = 1; L < kSegTileLevels; L++) {
        const int span = 1 << L;
        const int local = tid * span;             // first leaf (CTA-relative) of node tid at level L
        const int k = (blockIdx.x * kSegTile >> L) + tid;
        const bool live = local < kSegTile && k < seg_count(n, L);
        SegBox c;
        if (live) {
            c = sb[local];
            const int right = local + (span >> 1);
            if (blockIdx.x * kSegTile + right < n) c = seg_union(c, sb[right]);
        }
        __syncthreads();
        if (live) {
            sb[local] = c;
            put_box(seg, segf, seg_offset(n, L) + k, c);
        }
        __syncthreads();
    }
    // the levels above the CTAs, by the last CTA to finish
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (tid == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    int L = kSegTileLevels;  // the lowest level not built yet
    // through L2 while the level below holds more boxes than one tile
    for (; seg_count(n, L - 1) > kSegTile; L++) {
        const int cnt = seg_count(n, L), below = seg_count(n, L - 1);
        const int ob = seg_offset(n, L - 1), oc = seg_offset(n, L);
        for (int k = tid; k < cnt; k += blockDim.x) {
            SegBox c = seg_load_cg(seg + ob + 2 * k);
            if (2 * k + 1 < below) c = seg_union(c, seg_load_cg(seg + ob + 2 * k + 1));
            put_box(seg, segf, oc + k, c);
        }
        __threadfence();
        __syncthreads();
    }
    // the rest from one tile of the level below, in shared memory: node k of
    // m levels up sits at entry k 2^m of the tile
    const int cb = seg_count(n, L - 1);
    if (cb > 1) {
        if (tid < cb) sb[tid] = seg_load_cg(seg + seg_offset(n, L - 1) + tid);
        __syncthreads();
        for (int m = 1; (cb + (1 << (m - 1)) - 1) >> (m - 1) > 1; m++) {
            const int span = 1 << m;
            const int local = tid * span;
            const bool live = local < cb;
            SegBox c;
            if (live) {
                c = sb[local];
                const int right = local + (span >> 1);
                if (right < cb) c = seg_union(c, sb[right]);
            }
            __syncthreads();
            if (live) {
                sb[local] = c;
                put_box(seg, segf, seg_offset(n, L - 1 + m) + tid, c);
            }
            __syncthreads();
        }
    }
    if (tid == 0) *done = 0u;
}

void launch_bvh_build(const double* aabb, const int* sorted_idx, SegBox* seg, SegBoxF* segf, unsigned* done,
                      int ntri, cudaStream_t st) {
    if (ntri <= 0) return;
    k_mesh_tree<<<(ntri + kSegTile - 1) / kSegTile, kSegTile, 0, st>>>(aabb, sorted_idx, seg, segf, done, ntri);
}

// the segment tree's nodes: every level up to the root, and at least the
// levels one CTA writes
size_t bvh_scratch_bytes(int ntri) {
    if (ntri <= 0) return 0;
    const int levels = seg_levels(ntri) > kSegTileLevels ? seg_levels(ntri) : kSegTileLevels;
    return sizeof(SegBox) * (size_t)seg_offset(ntri, levels);
}

// FP32 copy of the triangles for the mixed-precision step kernel, and the
// low parts of its normal and corner-0 edges.
__global__ void k_trif(const TriRec* tri, TriRecF* out, TriLoF* lo, int ntri) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    const TriRec& T = tri[t];
    TriRecF F;
    TriLoF L;
    for (int k = 0; k < 3; k++) {
        split2(T.v0[k], F.v0h[k], F.v0l[k]);
        split2(T.n[k], F.n[k], L.nl[k]);
        split2(T.e01[k], F.e01[k], L.e01l[k]);
        split2(T.e02[k], F.e02[k], L.e02l[k]);
        F.e12[k] = (float)T.e12[k];
        L.pad[k] = 0.f;
    }
    F.d00 = (float)T.d00; F.d01 = (float)T.d01; F.d11 = (float)T.d11; F.denom = (float)T.denom;
    F.d00inv = (float)T.d00inv; F.d11inv = (float)T.d11inv; F.d22inv = (float)T.d22inv;
    F.i0 = T.i0; F.i1 = T.i1; F.i2 = T.i2; F.e0 = T.e0; F.e1 = T.e1; F.e2 = T.e2;
    F.pad = 0;
    out[t] = F;
    lo[t] = L;
}

void launch_trif(const TriRec* tri, TriRecF* out, TriLoF* lo, int ntri, cudaStream_t st) {
    if (ntri <= 0) return;
    k_trif<<<grid_for(ntri), kBlock, 0, st>>>(tri, out, lo, ntri);
}

// ===================================================================== probes
__global__ void k_dist_triangle(const TriRec* tri, const double* pos, const double* r, const int* t,
                                int m, double* out4, int* hit) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m) return;
    const double rr = r[q];
    const double rsq = rr * rr;
    const Feature f = closest_feature(pos[3 * q], pos[3 * q + 1], pos[3 * q + 2], rsq, tri[t[q]]);
    out4[4 * q + 0] = f.nx;
    out4[4 * q + 1] = f.ny;
    out4[4 * q + 2] = f.nz;
    out4[4 * q + 3] = f.dist;
    hit[q] = f.dist < 1e9 ? f.hit : -2;
}

void launch_dist_triangle(const TriRec* tri, const double* pos, const double* r, const int* t, int m,
                          double* out4, int* hit, cudaStream_t st) {
    if (m <= 0) return;
    k_dist_triangle<<<grid_for(m), kBlock, 0, st>>>(tri, pos, r, t, m, out4, hit);
}

}  // namespace gdem
