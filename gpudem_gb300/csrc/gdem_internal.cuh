// Internal device-side layout of the GB300 DEM engine.
//
// Per-particle data that neighbours gather lives in 16/32-byte records, so a
// neighbour costs three vector loads:
//   pos[i] = {x, y, z, r}           double4_32a (FP64 mode); mixed mode keeps the
//                                   float pairs posh/posl instead (SBank)
//   vel[i] = {vx, vy, vz, 1/m}      V4 (double4_32a in FP64 mode, float4 in mixed mode)
//   rot[i] = {wx, wy, wz, status}   V4; status 1 active, 0 inactive, 2 leaving the
//                                   box this step (still in this step's rebuild)
// Rows of variable length (Verlet list, wall list, contact history) are stored
// slot-major (element k of particle i at [k * n + i]) so a warp reads one slot
// of 32 consecutive particles in one transaction.
//
// Two state banks hold pos/vel/rot; the step kernel reads bank s and writes
// bank s^1.  Two property banks hold what moves only when the storage is
// Morton-reordered (material record, pId, contact history).  The control block
// (Ctl) in device memory says which bank is current, so captured CUDA graphs
// stay valid whatever the device decided at earlier steps.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

struct gdem_inlet;

namespace gdem {

constexpr int kBlock = 256;
constexpr unsigned kNoKey = 0xFFFFFFFFu;  // sort key of inactive particles (sorted last)
constexpr int kBvhStack = 64;
constexpr int kHintShift = 26;   // inner-row entries: index bits below, slot hint above

// ---------------------------------------------------------------- precision traits
struct FP64 {
    using real = double;
    using v4 = double4_32a;
    static constexpr bool mixed = false;
};
struct Mixed {
    using real = float;
    using v4 = float4;
    static constexpr bool mixed = true;   // FP32 contact math, compensated spring history
};

// One triangle of the wall mesh with everything dist_triangle reads
// (cpu_dem.cu:12-205), 256 bytes so a triangle is 8 full sectors.
struct __align__(16) TriRec {
    double n[3], d;
    double v0[3], v1[3], v2[3];
    double e01[3], e02[3], e12[3];
    double d00, d01, d11, denom, d00inv, d11inv, d22inv;
    int i0, i1, i2, e0, e1, e2;
};
static_assert(sizeof(TriRec) == 256, "TriRec must be 256 bytes");

// Mesh tree: a complete binary tree over the Morton-sorted triangles, kept
// level by level (level 0: the triangles' boxes in sorted order; node k of
// level L: the union of nodes 2k and 2k+1 of level L-1, so it covers sorted
// triangles [k 2^L, (k+1) 2^L)).  Every box contains the boxes below it, which
// is all a traversal needs.
struct __align__(16) SegBox {
    double lo[3], hi[3];
};
// the same box in FP32, rounded outwards (mixed-precision list build)
struct SegBoxF {
    float lo[3], hi[3];
};
constexpr int kSegMaxLevels = 32;
constexpr int kSegShift = 26;   // traversal stack entries: level << kSegShift | node

// Mixed-mode copy of a triangle: the first corner as a float pair, the rest
// in FP32 (128 bytes).
struct __align__(16) TriRecF {
    float v0h[3], v0l[3];
    float n[3];
    float e01[3], e02[3], e12[3];
    float d00, d01, d11, denom, d00inv, d11inv, d22inv;
    int i0, i1, i2, e0, e1, e2;
    int pad;
};
static_assert(sizeof(TriRecF) == 128, "TriRecF must be 128 bytes");

// Low parts of a mixed-mode triangle: with TriRecF's n, e01 and e02 they give
// the unit normal and the edges from the first corner as float pairs, for the
// overlap of a wall contact (48 bytes, read only for contacts).
struct __align__(16) TriLoF {
    float nl[3], e01l[3], e02l[3];
    float pad[3];
};
static_assert(sizeof(TriLoF) == 48, "TriLoF must be 48 bytes");

// Tries of a bounded wait on an mbarrier (bulk-copy completion) before the
// kernel gives up and sets GDEM_EW_TIMEOUT.
constexpr unsigned kSpinLimit = 1u << 22;

struct Ctl {
    int s;                    // state bank holding the current state
    int p;                    // property bank holding current properties/history
    unsigned refresh;         // set when some particle moved beyond the threshold
    unsigned error;           // GDEM_EW_* bits
    unsigned done[4];         // last-block counters (one per kernel family)
    unsigned long long steps;
    unsigned long long rebuilds;
    int max_nei, max_wall;
    int lists_valid;
    unsigned work;            // next sub-tile of the persistent step kernel (0 between steps)
    unsigned irefresh;        // mixed mode: the inner rows are to be rebuilt
    unsigned pad;
    unsigned long long inner_builds;
    unsigned wall_alloc;      // entries taken from the cell wall-candidate buffer (this rebuild)
    unsigned ncell_list;      // occupied cells listed in cell_list (this rebuild)
};

template <class T>
struct SBank {
    double4_32a* pos;        // FP64 mode: {x, y, z, r}
    typename T::v4* vel;
    typename T::v4* rot;
    // mixed mode: the positions and radii as unevaluated float pairs
    // x = hi + lo (|lo| <= ulp(hi)/2, about 48 significant bits), the only
    // copy of the positions: posh = {hi.xyz, r_hi}, with r_hi negated when
    // the particle is not active (status != 1), and posl = {lo.xyz, r_lo}.
    // hi + lo is exact in FP64; a pair's geometry is formed from the pairs
    // without cancellation error (pair_geometry in the mixed step).
    float4* posh;
    float4* posl;
    // mixed mode: low parts of the velocity and spin float pairs {lo.xyz, 0}
    float4* vell;
    float4* rotl;
};

// material record: linear model {k, etaconst, sqrt(m), 1/I};
// Hertz-Mindlin {k, etaconst, sqrt(m), 1/I}, or {mu, damping -2 sqrt(5/6) beta,
// sqrt(m), 1/I} once per-particle materials are set (gdem_set_particle_materials)
template <class T>
struct PBank {
    typename T::v4* mat;
    int* pid;
    int* nc;                         // particle contacts in history
    int* hid;                        // [hcap * n] contact partner: its pId (FP64 mode), its storage
                                     // index (mixed mode; remapped when the particles are reordered)
    typename T::real *hx, *hy, *hz;  // [hcap * n] tangential spring
    typename T::real *cx, *cy, *cz;  // [hcap * n] compensation terms (mixed mode)
    int* ncw;                        // wall contacts in history
    int* hwid;                       // [hwcap * n] triangle index
    typename T::real *hwx, *hwy, *hwz;
    typename T::real *cwx, *cwy, *cwz;
};

// Contact law constants.  Linear: per-particle k and etaconst from the
// material record (cpu_dem.cu:953).  Hertz-Mindlin (identical materials):
// E* = E/(2(1-nu^2)), G* = E/(4(1+nu)(2-nu)), beta = ln e/sqrt(ln^2 e + pi^2);
// kn = 4/3 E* sqrt(R* d), Sn = 2 E* sqrt(R* d), kt = St = 8 G* sqrt(R* d),
// damping -2 sqrt(5/6) beta sqrt(S m*).
struct Material {
    int model;              // 0 linear, 1 Hertz-Mindlin
    double mu;              // Coulomb coefficient
    double kn_c;            // 4/3 E*
    double sn_c;            // 2 E*
    double kt_c;            // 8 G*
    double damp_c;          // -2 sqrt(5/6) beta  (>= 0)
    double mu_roll;         // rolling friction coefficient (0: off)
};

template <class T>
struct View {
    int n;
    SBank<T> S[2];
    PBank<T> P[2];
    Ctl* ctl;
    // lists (rebuilt, not reordered)
    int *nei, *nnei, *neiw, *nneiw;
    double4_32a* ref;                // FP64 mode: {x, y, z, -} at the last rebuild
    float4* refh;                    // mixed mode: {hi.xyz, -} at the last rebuild
    float4* posf;                    // FP64 mode: FP32 positions for the list prefilter
    int nei_cap, wall_cap, hist_cap, histw_cap;
    // mixed mode, inner rows: the partners of each list row within
    // r_i + r_j + inner skin, in row order, and the high-part positions they
    // were taken at; the step kernels scan these instead of the list rows
    int* inn;
    int* ninn;
    int* innw;                       // ... and the wall-row triangles within r + inner skin
    int* ninnw;
    float4* refi;
    int inner_on;
    double inner_skin;
    float inner_skinf, inner_thresh_sqf;
    // inner rows with slot hints: an entry is the partner's storage index in
    // its low kHintShift bits and, above them, 1 + the partner's history slot
    // as last seen (0: not known); row_mask keeps the index (all ones when
    // entries carry no hints)
    unsigned row_mask;
    // per-step force/torque output
    double *fx, *fy, *fz, *tx, *ty, *tz;
    double* ftmp;                    // [6 * n] scratch for reordering the force outputs
    int store_forces;
    // sort scratch (ping-pong) and cell list
    uint32_t* keys[2];
    int* vals[2];
    int* inv;                        // mixed mode: old storage index -> new, at a reorder
    int* where;                      // storage index of each pId (set with the cell ranges)
    uint32_t* rs_hist;               // [256 * rs_blocks]
    uint32_t* rs_tot;                // [256]
    int rs_blocks;
    int *cell_start, *cell_end;
    int ncells, sizex, sizey, sizez;
    int reorder;
    // mesh
    const TriRec* tri;
    const TriRecF* trif;             // mixed mode
    const TriLoF* trilo;             // mixed mode
    float wall_delta;                // mixed mode: bound on the FP32 error of a wall distance (m)
    const SegBox* seg;               // mesh tree boxes, level by level
    const SegBoxF* segf;             // mixed mode: the same boxes in FP32
    const int* seg_tri;              // triangle of each level-0 node (Morton order)
    const double* tri_aabb;          // [6 * ntri] each triangle's box: min xyz, max xyz
    // wall candidates per occupied cell, indexed by the cell's first sorted
    // position: every triangle whose box comes within r_max + skin of the
    // cell, ascending; cw_cnt -1 sends the cell's particles through the tree
    int *cw_cnt, *cw_base, *cw_list;
    int* cell_list;                  // first sorted position of every occupied cell, ascending
                                     // (the cells the wall candidates are found for)
    int* cell_bc;                    // [blocks of kBlock sorted positions + 1] cell starts per block, scanned
    int cw_cap;                      // capacity of cw_list
    double cw_reach;                 // r_max + skin (+ the mixed rows' widening) + margin
    int seg_off[kSegMaxLevels];      // first box of each level
    int seg_top;                     // level of the root
    int ntri;
    // scalars
    Material mat;
    double dt;
    double gx, gy, gz;
    double minx, miny, minz, maxx, maxy, maxz;
    double invdx, invdy, invdz;
    // periodic x: the period Lx = maxx - minx, its half, and nxp cells across
    // it (cell x coordinates 1..nxp); in FP32 the period as a float pair
    int per_x, nxp;
    double Lx, halfLx;
    float Lxh, Lxl, halfLxf;
    float perf[2];                   // mixed mode: high-part x beyond which a centre may have left the period
    double skin, thresh_sq;
    float boxf[6];                   // mixed mode: box rounded outwards to FP32
    float nb_delta;                  // bound on |d_fp32 - d| of the list prefilter (m)
    int per_particle_mat;            // Hertz-Mindlin: mu and damping from mat.x, mat.y of each particle
    int kernel_variant;              // mixed step kernel: 0 default, 1 cooperative, 2 staged, 3 one-pass
    int occupancy;                   // mixed step kernel: resident CTAs per SM to size for (0 default)
    unsigned wait_tries;             // mixed step kernels: tries of each pipeline wait on a bulk copy
                                     // (kSpinLimit; GDEM_TEST_WAIT_TRIES lowers it to test the timeout path)
    // the scalars above rounded to FP32 once, for the mixed step
    float dtf, gxf, gyf, gzf, thresh_sqf;
    float muf, kn_cf, sn_cf, kt_cf, damp_cf, mu_rollf;
};

// Position {x, y, z, r} of particle i in FP64: the master in FP64 mode, the
// float pair hi + lo (exact in FP64) in mixed mode.
template <class T>
__device__ __forceinline__ double4_32a load_pos(const SBank<T>& S, int i) {
    if constexpr (T::mixed) {
        const float4 h = S.posh[i], l = S.posl[i];
        return make_double4_32a((double)h.x + (double)l.x, (double)h.y + (double)l.y,
                                (double)h.z + (double)l.z, (double)fabsf(h.w) + (double)l.w);
    } else {
        return S.pos[i];
    }
}

// ---------------------------------------------------------------- Morton
// 10-bit spread and interleave (x -> bit 2, y -> bit 1, z -> bit 0), the
// encoding of BoundingBox.h:125-135.
__host__ __device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
__host__ __device__ __forceinline__ uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    return (spread10(x) << 2) | (spread10(y) << 1) | spread10(z);
}
__host__ __device__ __forceinline__ uint32_t compact10(uint32_t v) {
    v &= 0x09249249u;
    v = (v | (v >> 2)) & 0x030C30C3u;
    v = (v | (v >> 4)) & 0x0300F00Fu;
    v = (v | (v >> 8)) & 0x030000FFu;
    v = (v | (v >> 16)) & 0x000003FFu;
    return v;
}

// Cell coordinate with the +1 ghost offset: floor((x - min) * invd) + 1
// (BoundingBox.cu:787-789).
__device__ __forceinline__ int cell_coord(double x, double mn, double invd) {
    return (int)floor((x - mn) * invd) + 1;
}

// ---------------------------------------------------------------- periodic x
// Cell x coordinate; with a periodic x every position lies in [minx, maxx)
// and the coordinate is kept in 1..nxp against rounding at the top face.
template <class T>
__device__ __forceinline__ int cell_x(const View<T>& v, double x) {
    int c = cell_coord(x, v.minx, v.invdx);
    if (v.per_x) c = c < 1 ? 1 : (c > v.nxp ? v.nxp : c);
    return c;
}
// Nearest-image x separation (the identity without a periodic x).
template <class T>
__device__ __forceinline__ double image_dx(const View<T>& v, double dx) {
    if (v.per_x) {
        if (dx > v.halfLx) dx -= v.Lx;
        else if (dx < -v.halfLx) dx += v.Lx;
    }
    return dx;
}
template <class T>
__device__ __forceinline__ float image_dxf(const View<T>& v, float dx) {
    if (v.per_x) {
        if (dx > v.halfLxf) dx -= v.Lxh;
        else if (dx < -v.halfLxf) dx += v.Lxh;
    }
    return dx;
}
// x of a sphere centre moved to the image nearest the triangle whose first
// corner is at x0 (triangles are narrower than a quarter period).
template <class T>
__device__ __forceinline__ double image_x_near(const View<T>& v, double x, double x0) {
    if (v.per_x) {
        const double d = x - x0;
        if (d > v.halfLx) x -= v.Lx;
        else if (d < -v.halfLx) x += v.Lx;
    }
    return x;
}

// ---------------------------------------------------------------- closest feature
struct Feature {
    double nx, ny, nz, dist;
    int hit;
};

// Sphere centre p against triangle t: the closest-feature classification of
// dist_triangle (cpu_dem.cu:12-205) with the contact radius squared `rsq`.
// FP64 operation order is kept term by term; compile without FMA contraction.
__device__ __forceinline__ Feature closest_feature(double px, double py, double pz, double rsq,
                                                   const TriRec& T) {
    Feature res;
    res.nx = 0.;
    res.ny = 0.;
    res.nz = 0.;
    res.dist = 1.e10;
    res.hit = -2;
    double dist = 0.;
    dist += T.n[0] * px;
    dist += T.n[1] * py;
    dist += T.n[2] * pz;
    dist += T.d;
    double distsq = dist * dist;
    if (distsq > rsq) return res;

    const double apx = px - T.v0[0], apy = py - T.v0[1], apz = pz - T.v0[2];
    const double d20 = apx * T.e01[0] + apy * T.e01[1] + apz * T.e01[2];
    const double d21 = apx * T.e02[0] + apy * T.e02[1] + apz * T.e02[2];
    const double v = (T.d11 * d20 - T.d01 * d21) * T.denom;
    const double w = (T.d00 * d21 - T.d01 * d20) * T.denom;
    const double u = 1.0 - v - w;
    if (u > 0. && v > 0. && w > 0.) {
        const double sign = dist < 0 ? -1.0 : 1.0;
        res.nx = sign * T.n[0];
        res.ny = sign * T.n[1];
        res.nz = sign * T.n[2];
        res.dist = sign * dist;
        res.hit = -1;
        return res;
    }
    double qx, qy, qz;  // closest point of the triangle
    int hit;
    if (v <= 0. && w <= 0.0) {
        qx = T.v0[0]; qy = T.v0[1]; qz = T.v0[2];
        hit = T.i0;
    } else if (u <= 0. && w <= 0.0) {
        qx = T.v1[0]; qy = T.v1[1]; qz = T.v1[2];
        hit = T.i1;
    } else if (u <= 0. && v <= 0.0) {
        qx = T.v2[0]; qy = T.v2[1]; qz = T.v2[2];
        hit = T.i2;
    } else if (u <= 0.0) {
        const double bx = px - T.v1[0], by = py - T.v1[1], bz = pz - T.v1[2];
        double t = (bx * T.e12[0] + by * T.e12[1] + bz * T.e12[2]) * T.d22inv;
        t = fmax(0., fmin(1.0, t));
        qx = T.v1[0] + t * T.e12[0];
        qy = T.v1[1] + t * T.e12[1];
        qz = T.v1[2] + t * T.e12[2];
        hit = T.e1;
    } else if (v <= 0.0) {
        double t = d21 * T.d11inv;
        t = fmax(0., fmin(1.0, t));
        qx = T.v0[0] + t * T.e02[0];
        qy = T.v0[1] + t * T.e02[1];
        qz = T.v0[2] + t * T.e02[2];
        hit = T.e2;
    } else {
        double t = d20 * T.d00inv;
        t = fmax(0., fmin(1.0, t));
        qx = T.v0[0] + t * T.e01[0];
        qy = T.v0[1] + t * T.e01[1];
        qz = T.v0[2] + t * T.e01[2];
        hit = T.e0;
    }
    res.nx = px - qx;
    res.ny = py - qy;
    res.nz = pz - qz;
    distsq = res.nx * res.nx + res.ny * res.ny + res.nz * res.nz;
    if (distsq < rsq) {
        res.dist = sqrt(distsq);
        const double inv = 1. / res.dist;
        res.nx = inv * res.nx;
        res.ny = inv * res.ny;
        res.nz = inv * res.nz;
    }
    res.hit = hit;
    return res;
}

// Squared distance test of a sphere of radius R around p against an AABB,
// sphereAABBOverlapNeighbor (BVH.cu:10-42).
__device__ __forceinline__ bool sphere_aabb(double px, double py, double pz, double Rsq,
                                            const double* lo, const double* hi) {
    double dx = 0.0, dy = 0.0, dz = 0.0;
    if (px < lo[0]) dx = lo[0] - px;
    else if (px > hi[0]) dx = px - hi[0];
    if (py < lo[1]) dy = lo[1] - py;
    else if (py > hi[1]) dy = py - hi[1];
    if (pz < lo[2]) dz = lo[2] - pz;
    else if (pz > hi[2]) dz = pz - hi[2];
    return (dx * dx + dy * dy + dz * dz) <= Rsq;
}

// ---------------------------------------------------------------- closest feature, FP32
struct FeatureF {
    float nx, ny, nz, dist;
    int hit;
    int kind;  // 0 face; 1, 2, 3 corner 0, 1, 2; 4 edge 1-2, 5 edge 0-2, 6 edge 0-1
    float t;   // edge parameter from the edge's first corner
};

// Closest feature of triangle T to the sphere centre (ph + pl) within radius^2
// rsq: the classification of dist_triangle (cpu_dem.cu:12-205) in FP32 on the
// corner-relative vector.
__device__ __forceinline__ FeatureF closest_feature_f(float3 ph, float3 pl, float rsq, const TriRecF& T) {
    FeatureF res;
    res.nx = res.ny = res.nz = 0.f;
    res.dist = 1.e10f;
    res.hit = -2;
    res.kind = 0;
    res.t = 0.f;
    const float ax = (ph.x - T.v0h[0]) + (pl.x - T.v0l[0]);
    const float ay = (ph.y - T.v0h[1]) + (pl.y - T.v0l[1]);
    const float az = (ph.z - T.v0h[2]) + (pl.z - T.v0l[2]);
    const float dist = T.n[0] * ax + T.n[1] * ay + T.n[2] * az;
    if (dist * dist > rsq) return res;
    const float d20 = ax * T.e01[0] + ay * T.e01[1] + az * T.e01[2];
    const float d21 = ax * T.e02[0] + ay * T.e02[1] + az * T.e02[2];
    const float v = (T.d11 * d20 - T.d01 * d21) * T.denom;
    const float w = (T.d00 * d21 - T.d01 * d20) * T.denom;
    const float u = 1.0f - v - w;
    if (u > 0.f && v > 0.f && w > 0.f) {
        const float sign = dist < 0.f ? -1.f : 1.f;
        res.nx = sign * T.n[0];
        res.ny = sign * T.n[1];
        res.nz = sign * T.n[2];
        res.dist = sign * dist;
        res.hit = -1;
        return res;
    }
    float rx, ry, rz;  // centre minus the closest point
    int hit, kind;
    float t = 0.f;
    if (v <= 0.f && w <= 0.f) {
        rx = ax; ry = ay; rz = az;
        hit = T.i0;
        kind = 1;
    } else if (u <= 0.f && w <= 0.f) {
        rx = ax - T.e01[0]; ry = ay - T.e01[1]; rz = az - T.e01[2];
        hit = T.i1;
        kind = 2;
    } else if (u <= 0.f && v <= 0.f) {
        rx = ax - T.e02[0]; ry = ay - T.e02[1]; rz = az - T.e02[2];
        hit = T.i2;
        kind = 3;
    } else if (u <= 0.f) {
        const float bx = ax - T.e01[0], by = ay - T.e01[1], bz = az - T.e01[2];
        t = (bx * T.e12[0] + by * T.e12[1] + bz * T.e12[2]) * T.d22inv;
        t = fmaxf(0.f, fminf(1.f, t));
        rx = bx - t * T.e12[0]; ry = by - t * T.e12[1]; rz = bz - t * T.e12[2];
        hit = T.e1;
        kind = 4;
    } else if (v <= 0.f) {
        t = d21 * T.d11inv;
        t = fmaxf(0.f, fminf(1.f, t));
        rx = ax - t * T.e02[0]; ry = ay - t * T.e02[1]; rz = az - t * T.e02[2];
        hit = T.e2;
        kind = 5;
    } else {
        t = d20 * T.d00inv;
        t = fmaxf(0.f, fminf(1.f, t));
        rx = ax - t * T.e01[0]; ry = ay - t * T.e01[1]; rz = az - t * T.e01[2];
        hit = T.e0;
        kind = 6;
    }
    res.kind = kind;
    res.t = t;
    const float dsq = rx * rx + ry * ry + rz * rz;
    if (dsq < rsq) {
        const float inv = rsqrtf(dsq);
        res.dist = dsq * inv;
        res.nx = rx * inv;
        res.ny = ry * inv;
        res.nz = rz * inv;
    }
    res.hit = hit;
    return res;
}

// "Last block of the grid" election without waiting: every block bumps a
// counter after its writes; the block that sees gridDim.x-1 runs the epilogue
// and resets the counter for the next launch.
__device__ __forceinline__ bool last_block(unsigned* counter) {
    __shared__ bool am_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned prev = atomicAdd(counter, 1u);
        am_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (am_last) __threadfence();
    return am_last;
}

// First slot of [0, n) whose bit is clear in `touched`, or n: the row length
// update_history (cpu_dem.cu:587-609) leaves.  Its swap-with-last loop never
// re-reads isContact after a swap, so every slot from the first lost contact
// on is dropped.
__device__ __forceinline__ int surviving(unsigned long long touched, int n) {
    const unsigned long long lost = ~touched;
    const int first = lost ? __ffsll((long long)lost) - 1 : 64;
    return first < n ? first : n;
}

// ---------------------------------------------------------------- launchers
// rebuild stages (gdem_rebuild.cu)
template <class T>
void launch_rebuild(const View<T>& v, cudaStream_t st, int force);
template <class T>
void launch_finalize_oob(const View<T>& v, cudaStream_t st);
// Triangle centroid Morton keys (and identity payload) from the records, as
// k_tri_precompute computes them.
void launch_tri_keys(const TriRec* rec, uint32_t* morton, int* idx, int ntri, const double* gmin,
                     const double* invrange, cudaStream_t st);
// Mesh tree of the Morton-sorted triangles (SegBox): every level's boxes in
// `seg` (bvh_scratch_bytes bytes) and their FP32 copies in `segf`.  `done` is
// a counter that must start at 0 (it is left at 0).
void launch_bvh_build(const double* aabb, const int* sorted_idx, SegBox* seg, SegBoxF* segf, unsigned* done,
                      int ntri, cudaStream_t st);
int seg_count_host(int n, int level);
int seg_offset_host(int n, int level);
int seg_levels(int n);
size_t bvh_scratch_bytes(int ntri);
void launch_tri_precompute(TriRec* rec, uint32_t* morton, int* idx, const double* vx,
                           const double* vy, const double* vz, const int* tv, const int* te,
                           const double* raw3, const double* dplane, int ntri, const double* gmin,
                           const double* invrange, cudaStream_t st);
void radix_sort_pairs(uint32_t* keys0, int* vals0, uint32_t* keys1, int* vals1, uint32_t* hist,
                      uint32_t* tot, int n, int nblocks, int first_pass, int npasses, cudaStream_t st);
int rs_blocks_for(int n);
void launch_dist_triangle(const TriRec* tri, const double* pos, const double* r, const int* t, int m,
                          double* out4, int* hit, cudaStream_t st);
void launch_trif(const TriRec* tri, TriRecF* out, TriLoF* lo, int ntri, cudaStream_t st);
// device-side particle initialisation (gdem_init.cu)
int init_particles_device(const gdem_inlet& in, int n, double* x, double* v, double* r, double* m, double* k,
                          double* eta, cudaStream_t st, std::string& msg);
// output frames (gdem_output.cu): write_frame_bin's payload built on the device
size_t frame_scratch_bytes(int n);
size_t frame_bytes(int n);
template <class T>
void launch_frame(const View<T>& v, void* scratch, char* frame, double length_factor, cudaStream_t st);
// inner rows (mixed mode with inner rows; gated on ctl->irefresh)
template <class T>
void launch_inner(const View<T>& v, cudaStream_t st);

// float pair split of an FP64 value: x == hi + lo to within 2^-48 |x|
__device__ __forceinline__ void split2(double x, float& hi, float& lo) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - (double)hi);
}
// step kernels (gdem_step_fp64.cu, gdem_step_mixed.cu)
void launch_step(const View<FP64>& v, cudaStream_t st, cudaGraphConditionalHandle cond, int use_cond);
void launch_step(const View<Mixed>& v, cudaStream_t st, cudaGraphConditionalHandle cond, int use_cond);
// The step kernel a launch uses and its launch shape.
struct StepLaunch {
    void* fn;
    dim3 grid, block;
    size_t smem;
};
// `reserve`: resident CTA slots the persistent step kernel leaves free for a
// graph branch that runs beside it (the mesh tree rebuild); the FP64 kernel
// is not persistent and ignores it.
StepLaunch step_launch(const View<FP64>& v, int reserve = 0);
StepLaunch step_launch(const View<Mixed>& v, int reserve = 0);
// CTA slots left free beside the per-step mesh tree rebuild
constexpr int kTreeReserve = 4;
// stats and probes (gdem_stats.cu)
template <class T>
void launch_stats(const View<T>& v, double* partials, int nblk, cudaStream_t st);
int stats_blocks(int n);
template <class T>
void launch_keys_probe(const View<T>& v, uint32_t* out, cudaStream_t st);

}  // namespace gdem
