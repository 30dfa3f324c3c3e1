// Device-side particle initialisation: the reference's "shuffle" inlet
// (initializeParticles, ParticleSystem.cu:189-340) without its O(N^2)
// rejection loop on the host, plus polydisperse radius distributions.
//
// Placement, all on the device and O(N):
//  * random: a maximal set of non-overlapping candidate centres by dart
//    throwing on a grid of cells of side 2 r_max / sqrt(3) (a cell holds at
//    most one centre).  Cells are visited in 125 phases (cell coordinates
//    modulo 5), so the cells of one phase are five cells apart and their
//    darts, which look two cells around, never race.  Then a random subset of
//    N candidates (a sort of random keys) becomes the particles: each centre
//    is uniform in the region, and no two are closer than 2 r_max.
//  * lattice: jittered simple-cubic sites of spacing 2 r_max (1 + gap) taken
//    in random order (a sort of random keys).
// Radii, velocities and jitter come from a counter-based generator
// (SplitMix64 of seed and index), so the result depends on the seed only.
//
// Compiled with -fmad=false: the masses and stiffnesses follow the reference's
// operation order (main.cu:67, ParticleSystem.cu:202, :301).
#include <math.h>

#include <string>

#include "../../include/gdem.h"
#include "gdem_internal.cuh"

namespace gdem {

namespace {

// SplitMix64 (Steele, Lea, Flood 2014): the output function of a 64-bit
// counter, here fed with seed, stream and index
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t rnd(uint64_t seed, uint64_t stream, uint64_t i) {
    return mix64(seed ^ mix64(stream * 0x100000001B3ull + i));
}
// uniform in [0, 1) with 53 bits
__device__ __forceinline__ double uni(uint64_t seed, uint64_t stream, uint64_t i) {
    return (double)(rnd(seed, stream, i) >> 11) * (1.0 / 9007199254740992.0);
}
// standard normal (Box-Muller)
__device__ __forceinline__ double gauss(uint64_t seed, uint64_t stream, uint64_t i) {
    const double u1 = 1.0 - uni(seed, stream, 2 * i), u2 = uni(seed, stream, 2 * i + 1);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

enum Stream : uint64_t { kDart = 1, kPick = 2, kRadius = 3, kVel = 4, kJitter = 5, kSite = 6 };

struct Grid {
    double lo[3], h;
    int nx, ny, nz;
};

// one phase of dart throwing: every empty cell of the phase tries `darts`
// uniform points in the cell and keeps the first with no centre within
// 2 r_max among the cells up to two away
__global__ void k_darts(Grid g, double4* cells, int phase, int round, int darts, double rmax, uint64_t seed,
                        const double* hi) {
    const int px = phase % 5, py = (phase / 5) % 5, pz = phase / 25;
    const int mx = (g.nx - px + 4) / 5, my = (g.ny - py + 4) / 5, mz = (g.nz - pz + 4) / 5;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)mx * my * mz) return;
    const int cx = px + 5 * (int)(t % mx), cy = py + 5 * (int)((t / mx) % my), cz = pz + 5 * (int)(t / ((long long)mx * my));
    const long long c = ((long long)cz * g.ny + cy) * g.nx + cx;
    if (cells[c].w != 0.0) return;
    const double d2min = 4.0 * rmax * rmax;
    for (int k = 0; k < darts; k++) {
        const uint64_t id = ((uint64_t)c * 64 + (uint64_t)round) * 64 + (uint64_t)k;
        const double x = g.lo[0] + (cx + uni(seed, kDart, 3 * id)) * g.h;
        const double y = g.lo[1] + (cy + uni(seed, kDart, 3 * id + 1)) * g.h;
        const double z = g.lo[2] + (cz + uni(seed, kDart, 3 * id + 2)) * g.h;
        if (x > hi[0] || y > hi[1] || z > hi[2]) continue;  // the last cells stick out of the region
        bool free = true;
        for (int dz = -2; dz <= 2 && free; dz++) {
            const int zz = cz + dz;
            if (zz < 0 || zz >= g.nz) continue;
            for (int dy = -2; dy <= 2 && free; dy++) {
                const int yy = cy + dy;
                if (yy < 0 || yy >= g.ny) continue;
                for (int dx = -2; dx <= 2; dx++) {
                    const int xx = cx + dx;
                    if (xx < 0 || xx >= g.nx) continue;
                    const double4 o = cells[((long long)zz * g.ny + yy) * g.nx + xx];
                    if (o.w == 0.0) continue;
                    const double ex = x - o.x, ey = y - o.y, ez = z - o.z;
                    if (ex * ex + ey * ey + ez * ez < d2min) {
                        free = false;
                        break;
                    }
                }
            }
        }
        if (free) {
            cells[c] = make_double4(x, y, z, 1.0);
            return;
        }
    }
}

// random keys of the candidates (filled cells) for the pick of N of them;
// empty cells get the largest key and sort last
__global__ void k_cell_keys(const double4* cells, long long ncell, uint32_t* keys, int* vals, uint64_t seed) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    keys[c] = cells[c].w != 0.0 ? (uint32_t)(rnd(seed, kPick, (uint64_t)c) >> 33) : 0xFFFFFFFFu;
    vals[c] = (int)c;
}

// random keys of the lattice sites
__global__ void k_site_keys(long long nsite, uint32_t* keys, int* vals, uint64_t seed) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsite) return;
    keys[s] = (uint32_t)(rnd(seed, kSite, (uint64_t)s) >> 32);
    vals[s] = (int)s;
}

__global__ void k_count_filled(const double4* cells, long long ncell, unsigned long long* count) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool f = c < ncell && cells[c].w != 0.0;
    const unsigned b = __ballot_sync(0xffffffffu, f);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(count, (unsigned long long)__popc(b));
}

__device__ double sample_radius(const gdem_inlet& in, uint64_t seed, int i) {
    switch (in.radius_dist) {
        case GDEM_RADIUS_UNIFORM:
            return in.r_a + uni(seed, kRadius, (uint64_t)i) * (in.r_b - in.r_a);
        case GDEM_RADIUS_LOGNORMAL: {
            const double r = in.r_a * exp(in.r_b * gauss(seed, kRadius, (uint64_t)i));
            return fmin(fmax(r, in.r_c), in.r_d);
        }
        case GDEM_RADIUS_BIDISPERSE:
            return uni(seed, kRadius, (uint64_t)i) < in.r_c ? in.r_a : in.r_b;
        default:
            return in.r_a;
    }
}

// The particles in the reference layout: centre i from candidate / site
// vals[i], its radius, mass (rho * 3.14 * r^3 * 4/3 in main.cu:67's order),
// linear stiffness and damping constant (ParticleSystem.cu:202, :301) and
// velocity.
// log_res is ln(restitution) from the host's C library, the log the
// reference's initializeParticles calls, so that the damping constant matches
// it bit for bit (the device log may round differently).
__global__ void k_make_particles(gdem_inlet in, int n, double rmax, const int* vals, const double4* cells,
                                 long long sx, long long sy, double* x, double* v, double* r, double* m, double* k,
                                 double* eta, double log_res) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t seed = in.seed;
    double px, py, pz;
    if (in.placement == GDEM_PLACE_LATTICE) {
        const long long s = vals[i];
        const double a = 2.0 * rmax * (1.0 + in.gap);
        const long long iz = s % sx;  // z fastest, as scenes.lattice_packing
        const long long iy = (s / sx) % sy;
        const long long ix = s / (sx * sy);
        px = in.box_min[0] + rmax + ix * a + (uni(seed, kJitter, 3 * (uint64_t)i) - 0.5) * (in.gap * rmax);
        py = in.box_min[1] + rmax + iy * a + (uni(seed, kJitter, 3 * (uint64_t)i + 1) - 0.5) * (in.gap * rmax);
        pz = in.box_min[2] + rmax + iz * a + (uni(seed, kJitter, 3 * (uint64_t)i + 2) - 0.5) * (in.gap * rmax);
    } else {
        const double4 c = cells[vals[i]];
        px = c.x;
        py = c.y;
        pz = c.z;
    }
    x[3 * i] = px;
    x[3 * i + 1] = py;
    x[3 * i + 2] = pz;
    const double ri = sample_radius(in, seed, i);
    r[i] = ri;
    m[i] = (((((in.density * 3.14) * ri) * ri) * ri) * 4.0) / 3.0;
    const double E = in.youngs_modulus;
    const double ki = 4. / 3. * (E * 0.5) * sqrt(ri * 0.5) * sqrt(0.05 * ri);
    k[i] = ki;
    const double le = log_res;
    eta[i] = -2. * le * sqrt(ki / (3.1415 * 3.1415 + le * le));
    for (int a = 0; a < 3; a++)
        v[3 * i + a] = in.velocity[a] + (in.velocity_sigma > 0. ? in.velocity_sigma * gauss(seed, kVel, 3 * (uint64_t)i + a) : 0.);
}

}  // namespace

double inlet_rmax(const gdem_inlet& in) {
    switch (in.radius_dist) {
        case GDEM_RADIUS_UNIFORM: return in.r_a > in.r_b ? in.r_a : in.r_b;
        case GDEM_RADIUS_LOGNORMAL: return in.r_d;
        case GDEM_RADIUS_BIDISPERSE: return in.r_a > in.r_b ? in.r_a : in.r_b;
        default: return in.r_a;
    }
}

// Place n particles on the device; x, v [3n], r, m, k, eta [n] are device
// arrays.  Returns 0, or GDEM_ERR_RANGE when the region holds fewer than n.
int init_particles_device(const gdem_inlet& in, int n, double* x, double* v, double* r, double* m, double* k,
                          double* eta, cudaStream_t st, std::string& msg) {
    const double rmax = inlet_rmax(in);
    double* dhi = nullptr;
    uint32_t *keys0 = nullptr, *keys1 = nullptr, *hist = nullptr, *tot = nullptr;
    int *vals0 = nullptr, *vals1 = nullptr;
    double4* cells = nullptr;
    unsigned long long* count = nullptr;
    long long nitems = 0, sx = 0, sy = 0;
    int rc = GDEM_OK;
    auto fail = [&](int code, const std::string& s) {
        msg = s;
        rc = code;
    };
#define CKI(call)                                                        \
    do {                                                                 \
        cudaError_t e_ = (call);                                         \
        if (e_ != cudaSuccess) {                                         \
            fail(GDEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
            goto done;                                                   \
        }                                                                \
    } while (0)
    {
        const int B = 256;
        if (in.placement == GDEM_PLACE_LATTICE) {
            const double a = 2.0 * rmax * (1.0 + in.gap);
            long long dims[3];
            for (int q = 0; q < 3; q++) {
                const double ext = in.box_max[q] - in.box_min[q] - 2 * rmax;
                dims[q] = ext < 0 ? 0 : (long long)floor(ext / a) + 1;
            }
            nitems = dims[0] * dims[1] * dims[2];
            sx = dims[2];
            sy = dims[1];
            if (nitems < n) {
                fail(GDEM_ERR_RANGE, "init: the lattice region holds fewer sites than particles");
                goto done;
            }
            if (nitems > (1ll << 30)) {
                fail(GDEM_ERR_RANGE, "init: more than 2^30 lattice sites");
                goto done;
            }
        } else {
            Grid g;
            g.h = 2.0 * rmax / sqrt(3.0) * (1.0 - 1e-12);
            long long dims[3];
            for (int q = 0; q < 3; q++) {
                g.lo[q] = in.box_min[q];
                const double ext = in.box_max[q] - in.box_min[q];
                dims[q] = ext <= 0 ? 0 : (long long)ceil(ext / g.h);
            }
            g.nx = (int)dims[0];
            g.ny = (int)dims[1];
            g.nz = (int)dims[2];
            nitems = dims[0] * dims[1] * dims[2];
            if (nitems <= 0 || nitems > (1ll << 30)) {
                fail(GDEM_ERR_RANGE, "init: the region is empty or needs more than 2^30 cells");
                goto done;
            }
            CKI(cudaMalloc(&dhi, 3 * sizeof(double)));
            CKI(cudaMemcpyAsync(dhi, in.box_max, 3 * sizeof(double), cudaMemcpyHostToDevice, st));
            CKI(cudaMalloc(&cells, sizeof(double4) * nitems));
            CKI(cudaMemsetAsync(cells, 0, sizeof(double4) * nitems, st));
            const int rounds = 3, darts = 8;
            for (int rd = 0; rd < rounds; rd++)
                for (int ph = 0; ph < 125; ph++) {
                    const long long per = (long long)((g.nx + 4) / 5) * ((g.ny + 4) / 5) * ((g.nz + 4) / 5);
                    k_darts<<<(unsigned)((per + B - 1) / B), B, 0, st>>>(g, cells, ph, rd, darts, rmax, in.seed, dhi);
                }
            CKI(cudaGetLastError());
            CKI(cudaMalloc(&count, sizeof(unsigned long long)));
            CKI(cudaMemsetAsync(count, 0, sizeof(unsigned long long), st));
            k_count_filled<<<(unsigned)((nitems + B - 1) / B), B, 0, st>>>(cells, nitems, count);
            unsigned long long got = 0;
            CKI(cudaMemcpyAsync(&got, count, sizeof(got), cudaMemcpyDeviceToHost, st));
            CKI(cudaStreamSynchronize(st));
            if (got < (unsigned long long)n) {
                fail(GDEM_ERR_RANGE, "init: the region holds only " + std::to_string(got) +
                                         " non-overlapping particles");
                goto done;
            }
        }
        // a random order of the candidates or sites: sort random keys
        const int nb = rs_blocks_for((int)nitems);
        CKI(cudaMalloc(&keys0, sizeof(uint32_t) * nitems));
        CKI(cudaMalloc(&keys1, sizeof(uint32_t) * nitems));
        CKI(cudaMalloc(&vals0, sizeof(int) * nitems));
        CKI(cudaMalloc(&vals1, sizeof(int) * nitems));
        CKI(cudaMalloc(&hist, sizeof(uint32_t) * 256 * (size_t)nb));
        CKI(cudaMalloc(&tot, sizeof(uint32_t) * 256));
        if (in.placement == GDEM_PLACE_LATTICE)
            k_site_keys<<<(unsigned)((nitems + B - 1) / B), B, 0, st>>>(nitems, keys0, vals0, in.seed);
        else
            k_cell_keys<<<(unsigned)((nitems + B - 1) / B), B, 0, st>>>(cells, nitems, keys0, vals0, in.seed);
        radix_sort_pairs(keys0, vals0, keys1, vals1, hist, tot, (int)nitems, nb, 0, 4, st);
        k_make_particles<<<(n + B - 1) / B, B, 0, st>>>(in, n, rmax, vals0, cells, sx, sy, x, v, r, m, k, eta,
                                                         std::log(in.restitution));
        CKI(cudaGetLastError());
        CKI(cudaStreamSynchronize(st));
    }
done:
#undef CKI
    cudaFree(dhi);
    cudaFree(cells);
    cudaFree(count);
    cudaFree(keys0);
    cudaFree(keys1);
    cudaFree(vals0);
    cudaFree(vals1);
    cudaFree(hist);
    cudaFree(tot);
    return rc;
}

}  // namespace gdem
