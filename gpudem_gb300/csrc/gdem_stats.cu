// Per-block reductions of the parity observables (kinetic energy, contact
// and list counts, coordination, packing, maximum overlap), the Morton-key
// probe and the pId-order position gather used by exports.  The reference has
// only an unused kineticEnergy (cpu_dem.cu:1554); these reductions are
// deterministic: each block owns a fixed index range and the host adds the
// block partials in block order.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gdem_internal.cuh"

namespace gdem {

constexpr int kStatBlocks = 1024;
constexpr int kNStat = 16;

int stats_blocks(int n) {
    const int g = (n + kBlock - 1) / kBlock;
    return g < kStatBlocks ? (g > 0 ? g : 1) : kStatBlocks;
}

template <class T>
__global__ void __launch_bounds__(kBlock) k_stats(View<T> v, double* partials) {
    const Ctl* ctl = v.ctl;
    const SBank<T> S = v.S[ctl->s];
    const PBank<T> P = v.P[ctl->p];
    double acc[kNStat];
    for (int k = 0; k < kNStat; k++) acc[k] = 0.;
    for (int k = 7; k < 10; k++) acc[k] = 1e300;
    for (int k = 10; k < 13; k++) acc[k] = -1e300;
    const int n = v.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const auto w = S.rot[i];
        if (w.w != 1) continue;
        const double4_32a p = load_pos(S, i);
        const auto ve = S.vel[i];
        const double r = p.w;
        const double m = 1. / (double)ve.w, I = 1. / (double)P.mat[i].w;
        const double vv = (double)ve.x * ve.x + (double)ve.y * ve.y + (double)ve.z * ve.z;
        const double ww = (double)w.x * w.x + (double)w.y * w.y + (double)w.z * w.z;
        acc[0] += 1.;
        acc[1] += v.nnei[i];
        acc[2] += v.nneiw[i];
        acc[3] += P.nc[i];
        acc[4] += P.ncw[i];
        acc[5] += 0.5 * m * vv + 0.5 * I * ww;
        acc[6] += 4.0 / 3.0 * 3.141592653589793 * r * r * r;
        acc[7] = fmin(acc[7], p.x - r);
        acc[8] = fmin(acc[8], p.y - r);
        acc[9] = fmin(acc[9], p.z - r);
        acc[10] = fmax(acc[10], p.x + r);
        acc[11] = fmax(acc[11], p.y + r);
        acc[12] = fmax(acc[12], p.z + r);
        if (v.inner_on) {
            acc[14] += v.ninn[i];
            acc[15] += v.ninnw[i];
        }
        const int nn = v.nnei[i];
        for (int k = 0; k < nn; k++) {
            const int j = v.nei[(size_t)k * n + i];
            if (S.rot[j].w != 1) continue;
            const double4_32a q = load_pos(S, j);
            const double dx = image_dx(v, p.x - q.x), dy = p.y - q.y, dz = p.z - q.z;
            const double R = r + q.w;
            const double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 < R * R) acc[13] = fmax(acc[13], (R - sqrt(d2)) / (2. * r));
        }
    }
    __shared__ double sm[kNStat][kBlock];
    for (int k = 0; k < kNStat; k++) sm[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int o = kBlock / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            for (int k = 0; k < 7; k++) sm[k][threadIdx.x] += sm[k][threadIdx.x + o];
            for (int k = 7; k < 10; k++) sm[k][threadIdx.x] = fmin(sm[k][threadIdx.x], sm[k][threadIdx.x + o]);
            for (int k = 10; k < 14; k++) sm[k][threadIdx.x] = fmax(sm[k][threadIdx.x], sm[k][threadIdx.x + o]);
            sm[14][threadIdx.x] += sm[14][threadIdx.x + o];
            sm[15][threadIdx.x] += sm[15][threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x < kNStat) partials[16 * blockIdx.x + threadIdx.x] = sm[threadIdx.x][0];
}

template <class T>
void launch_stats(const View<T>& v, double* partials, int nblk, cudaStream_t st) {
    k_stats<T><<<nblk, kBlock, 0, st>>>(v, partials);
}

// Morton key of every stored particle into `out` (the formula of k_keys, for
// particles active from the caller's point of view).
template <class T>
__global__ void k_keys_probe(View<T> v, uint32_t* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.n) return;
    const SBank<T> S = v.S[v.ctl->s];
    uint32_t key = kNoKey;
    if (S.rot[i].w == 1) {
        const double4_32a p = load_pos(S, i);
        const int cx = cell_x(v, p.x);
        const int cy = cell_coord(p.y, v.miny, v.invdy);
        const int cz = cell_coord(p.z, v.minz, v.invdz);
        key = morton3((uint32_t)cx, (uint32_t)cy, (uint32_t)cz);
    }
    out[i] = key;
}

template <class T>
void launch_keys_probe(const View<T>& v, uint32_t* out, cudaStream_t st) {
    k_keys_probe<T><<<(v.n + kBlock - 1) / kBlock, kBlock, 0, st>>>(v, out);
}

// Positions in pId order, xyz-interleaved (the reference layout of x[]).
template <class T>
__global__ void k_gather_positions(View<T> v, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.n) return;
    const double4_32a p = load_pos(v.S[v.ctl->s], i);
    const int q = v.P[v.ctl->p].pid[i];
    out[3 * (size_t)q + 0] = p.x;
    out[3 * (size_t)q + 1] = p.y;
    out[3 * (size_t)q + 2] = p.z;
}

template <class T>
void launch_gather_positions(const View<T>& v, double* out, cudaStream_t st) {
    k_gather_positions<T><<<(v.n + kBlock - 1) / kBlock, kBlock, 0, st>>>(v, out);
}

template void launch_stats<FP64>(const View<FP64>&, double*, int, cudaStream_t);
template void launch_stats<Mixed>(const View<Mixed>&, double*, int, cudaStream_t);
template void launch_keys_probe<FP64>(const View<FP64>&, uint32_t*, cudaStream_t);
template void launch_keys_probe<Mixed>(const View<Mixed>&, uint32_t*, cudaStream_t);
template void launch_gather_positions<FP64>(const View<FP64>&, double*, cudaStream_t);
template void launch_gather_positions<Mixed>(const View<Mixed>&, double*, cudaStream_t);

}  // namespace gdem
