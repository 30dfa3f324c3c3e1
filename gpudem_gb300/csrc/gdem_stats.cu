// Per-block reductions of the parity observables (kinetic energy, contact
// and list counts, coordination, packing, maximum overlap) and the Morton-key
// probe.  The reference has only an unused kineticEnergy (cpu_dem.cu:1554);
// these reductions are deterministic: each block owns a fixed index range and
// the host adds the block partials in block order.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gdem_internal.cuh"

namespace gdem {

constexpr int kStatBlocks = 1024;
constexpr int kNStat = 14;

int stats_blocks(int n) {
    const int g = (n + kBlock - 1) / kBlock;
    return g < kStatBlocks ? (g > 0 ? g : 1) : kStatBlocks;
}

__global__ void __launch_bounds__(kBlock) k_stats(View v, double* partials) {
    const Ctl* ctl = v.ctl;
    const SBank S = v.S[ctl->s];
    const PBank P = v.P[ctl->p];
    double acc[kNStat];
    for (int k = 0; k < kNStat; k++) acc[k] = 0.;
    for (int k = 7; k < 10; k++) acc[k] = 1e300;
    for (int k = 10; k < 13; k++) acc[k] = -1e300;
    const int n = v.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (S.active[i] != 1) continue;
        const double x = S.x[i], y = S.y[i], z = S.z[i], r = P.r[i];
        const double m = 1. / P.invm[i], I = 1. / P.invmoi[i];
        const double vv = S.vx[i] * S.vx[i] + S.vy[i] * S.vy[i] + S.vz[i] * S.vz[i];
        const double ww = S.wx[i] * S.wx[i] + S.wy[i] * S.wy[i] + S.wz[i] * S.wz[i];
        acc[0] += 1.;
        acc[1] += v.nnei[i];
        acc[2] += v.nneiw[i];
        acc[3] += P.nc[i];
        acc[4] += P.ncw[i];
        acc[5] += 0.5 * m * vv + 0.5 * I * ww;
        acc[6] += 4.0 / 3.0 * 3.141592653589793 * r * r * r;
        acc[7] = fmin(acc[7], x - r);
        acc[8] = fmin(acc[8], y - r);
        acc[9] = fmin(acc[9], z - r);
        acc[10] = fmax(acc[10], x + r);
        acc[11] = fmax(acc[11], y + r);
        acc[12] = fmax(acc[12], z + r);
        const int nn = v.nnei[i];
        for (int k = 0; k < nn; k++) {
            const int j = v.nei[(size_t)k * n + i];
            if (S.active[j] != 1) continue;
            const double dx = x - S.x[j], dy = y - S.y[j], dz = z - S.z[j];
            const double R = r + P.r[j];
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
        }
        __syncthreads();
    }
    if (threadIdx.x < kNStat) partials[16 * blockIdx.x + threadIdx.x] = sm[threadIdx.x][0];
}

void launch_stats(const View& v, double* partials, int nblk, cudaStream_t st) {
    k_stats<<<nblk, kBlock, 0, st>>>(v, partials);
}

// Morton key of every stored particle into `out` (same formula as k_keys).
__global__ void k_keys_probe(View v, uint32_t* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.n) return;
    const SBank S = v.S[v.ctl->s];
    uint32_t key = kNoKey;
    if (S.active[i] == 1) {
        const int cx = cell_coord(S.x[i], v.minx, v.invdx);
        const int cy = cell_coord(S.y[i], v.miny, v.invdy);
        const int cz = cell_coord(S.z[i], v.minz, v.invdz);
        key = morton3((uint32_t)cx, (uint32_t)cy, (uint32_t)cz);
    }
    out[i] = key;
}

void launch_keys_probe(const View& v, uint32_t* out, cudaStream_t st) {
    k_keys_probe<<<(v.n + kBlock - 1) / kBlock, kBlock, 0, st>>>(v, out);
}

}  // namespace gdem
