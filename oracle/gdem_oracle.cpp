// CPU restatement of gpudem's step path — TEST INFRASTRUCTURE ONLY.
//
// This is the oracle the CUDA engine is checked against on machines where the
// reference itself cannot be built (the GPU host), and the CPU baseline timed
// by bench.py.  It is never linked into, called by, or used as a fallback of
// the product (gpudem_gb300/_build/libgdem.so).  It is pinned bit for bit to
// the unmodified reference by tests/test_oracle.py against tests/golden/*.npz.
//
// It restates, in the reference's own data layout (xyz-interleaved vectors,
// MAX_NEI-strided rows) and FP64 operation order (compile without FMA
// contraction):
//   mesh ingestion     TriangleMesh.cu:363-752 (weld, sort3, edges, precompute,
//                      centroid Morton keys, radixSortUint32)
//   BVH                BVH.cu:712-787 (median split over the Morton order)
//   box / cells        BoundingBox.cu:364-446, update_pList :839-894,
//                      update_pList_withSort :664-731, morton3D BoundingBox.h:125
//   Verlet lists       update_neighborlist BoundingBox.cu:526-587
//   wall lists         update_neighborlist_wall BVH.cu:576-625
//   step               cpu_dem_verlet_verlet cpu_dem.cu:1593-1668 and
//                      checkOoB cpu_dem.cu:1575-1589, as main.cu:302-316 calls them
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <unordered_map>
#include <vector>

namespace {

constexpr int K = 100;  // MAX_NEI, hardCodedParameters.h:3

struct V3 {
    double x, y, z;
};
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 scale(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

inline uint32_t spread(uint32_t v) {
    v &= 0x000003ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
inline uint32_t morton(uint32_t x, uint32_t y, uint32_t z) { return (spread(x) << 2) | (spread(y) << 1) | spread(z); }

// LSB radix sort, 4 passes of 8 bits, stable (radixSortUint32, BoundingBox.cu:33)
void lsb_sort(std::vector<uint32_t>& key, std::vector<int>& idx) {
    const size_t n = key.size();
    std::vector<uint32_t> k2(n);
    std::vector<int> i2(n);
    for (int pass = 0; pass < 4; pass++) {
        const int sh = 8 * pass;
        size_t cnt[256] = {0};
        for (size_t i = 0; i < n; i++) cnt[(key[i] >> sh) & 0xFF]++;
        size_t run = 0;
        for (int d = 0; d < 256; d++) {
            const size_t c = cnt[d];
            cnt[d] = run;
            run += c;
        }
        for (size_t i = 0; i < n; i++) {
            const size_t pos = cnt[(key[i] >> sh) & 0xFF]++;
            k2[pos] = key[i];
            i2[pos] = idx[i];
        }
        key.swap(k2);
        idx.swap(i2);
    }
}

struct Mesh {
    int nTri = 0, nShift = 0;
    std::vector<double> mx, my, mz;  // welded vertices
    std::vector<int> i0, i1, i2, e0, e1, e2;
    std::vector<double> nx, ny, nz, d, e01x, e01y, e01z, e02x, e02y, e02z, e12x, e12y, e12z;
    std::vector<double> d00, d00inv, d01, d11, d11inv, d22, d22inv, denom;
    std::vector<double> minx, miny, minz, maxx, maxy, maxz, cx, cy, cz;
    double g[6];
    std::vector<uint32_t> key;  // sorted centroid keys
    std::vector<int> sorted;    // their permutation
};

struct Bvh {
    std::vector<double> lo[3], hi[3];
    std::vector<int> left, right, tri;
    int nodes = 0;
};

struct Contact {
    V3 fn, vn, vt, n;
    double eta;   // tangential damping (the linear law reuses the normal one)
    double kt;    // tangential stiffness (the linear law uses k_i)
    double Rstar; // effective radius (rolling resistance)
};

struct Feature {
    V3 n;
    double dist;
    int hit;
};

struct Scene {
    int N = 0;
    double dt = 0., mu = 0., g[3] = {0, 0, 0};
    // contact law: 0 linear (the reference's), 1 Hertz-Mindlin (restated from
    // the published law; the reference has none)
    int model = 0;
    double kn_c = 0., sn_c = 0., kt_c = 0., damp_c = 0., mu_roll = 0.;
    // Hertz-Mindlin friction and damping per particle (several scenes packed
    // into one, each with its own material); empty: the scene-wide values.
    // Particle i's own values enter its contacts, as in the engine.
    std::vector<double> mu_p, damp_p;
    double mu_of(int i) const { return mu_p.empty() ? mu : mu_p[i]; }
    double damp_of(int i) const { return damp_p.empty() ? damp_c : damp_p[i]; }
    std::vector<double> x, v, a, f, w, anga, mom, r, rsq, invr, k, m, sqrtm, invm, moi, invmoi, eta;
    std::vector<int> active, pId;
    std::vector<double> hx, hy, hz, hwx, hwy, hwz;
    std::vector<int> hid, hwid, vore, isC, isCW, nc, ncw;
    std::vector<int> cellx, cellId;
    std::vector<double> refx, refy, refz;
    std::vector<int> nei, nnei, neiw, nneiw;
    // box
    double bmin[3], bmax[3], dx, inv, skin, thresh, threshSq;
    // periodic x (an extension; the reference has none): [bmin[0], bmax[0])
    // is one period L, nxp cells of 1/invx across it
    int per_x = 0, nxp = 0;
    double L = 0., halfL = 0., invx = 0.;
    int size[3], ncells;
    std::vector<int> pNum, pStart, pList, cellOff;
    Mesh mesh;
    Bvh bvh;
    long steps = 0, rebuilds = 0;
};

// ------------------------------------------------------------------ mesh
struct QKey {
    long long a, b, c;
    bool operator==(const QKey& o) const { return a == o.a && b == o.b && c == o.c; }
};
struct QHash {
    size_t operator()(const QKey& q) const {
        return std::hash<long long>()(q.a) ^ (std::hash<long long>()(q.b) * 31) ^ (std::hash<long long>()(q.c) * 131);
    }
};

void ingest(Mesh& M, const double* tris, int T, const int* files, int nfiles) {
    M.nTri = T;
    M.nShift = 3 * T;
    auto rs = [&](std::vector<double>& v) { v.assign(T, 0.); };
    for (auto* v : {&M.nx, &M.ny, &M.nz, &M.d, &M.e01x, &M.e01y, &M.e01z, &M.e02x, &M.e02y, &M.e02z, &M.e12x,
                    &M.e12y, &M.e12z, &M.d00, &M.d00inv, &M.d01, &M.d11, &M.d11inv, &M.d22, &M.d22inv,
                    &M.denom, &M.minx, &M.miny, &M.minz, &M.maxx, &M.maxy, &M.maxz, &M.cx, &M.cy, &M.cz})
        rs(*v);
    for (auto* v : {&M.i0, &M.i1, &M.i2, &M.e0, &M.e1, &M.e2}) v->assign(T, 0);
    for (int k = 0; k < 3; k++) {
        M.g[k] = 1e300;
        M.g[3 + k] = -1e300;
    }
    std::vector<int> fl;
    if (files && nfiles > 0)
        fl.assign(files, files + nfiles);
    else
        fl.push_back(T);
    std::unordered_map<unsigned long long, int> edges;
    int ne = 0, t = 0;
    for (int f : fl) {
        std::unordered_map<QKey, int, QHash> weld;
        for (int q = 0; q < f; q++, t++) {
            int id[3];
            double X = 0, Y = 0, Z = 0;
            for (int c = 0; c < 3; c++) {
                X = tris[9 * t + 3 * c];
                Y = tris[9 * t + 3 * c + 1];
                Z = tris[9 * t + 3 * c + 2];
                QKey key{llround(X / 1e-9), llround(Y / 1e-9), llround(Z / 1e-9)};
                auto it = weld.find(key);
                if (it == weld.end()) {
                    id[c] = (int)M.mx.size();
                    weld.emplace(key, id[c]);
                    M.mx.push_back(X);
                    M.my.push_back(Y);
                    M.mz.push_back(Z);
                } else {
                    id[c] = it->second;
                }
            }
            // X, Y, Z now hold the third corner as read (the plane offset uses it)
            int a = id[0], b = id[1], c = id[2], s;
            if (a > b) { s = a; a = b; b = s; }
            if (b > c) { s = b; b = c; c = s; }
            if (a > b) { s = a; a = b; b = s; }
            const int pr[3][2] = {{a, b}, {b, c}, {a, c}};
            int eid[3];
            for (int e = 0; e < 3; e++) {
                const unsigned long long kk = ((unsigned long long)(unsigned)pr[e][0] << 32) | (unsigned)pr[e][1];
                auto it = edges.find(kk);
                if (it == edges.end()) {
                    eid[e] = ne++;
                    edges.emplace(kk, eid[e]);
                } else {
                    eid[e] = it->second;
                }
            }
            M.e0[t] = eid[0] + M.nShift;
            M.e1[t] = eid[1] + M.nShift;
            M.e2[t] = eid[2] + M.nShift;
            const V3 p0{M.mx[a], M.my[a], M.mz[a]}, p1{M.mx[b], M.my[b], M.mz[b]}, p2{M.mx[c], M.my[c], M.mz[c]};
            const V3 e01 = sub(p1, p0), e02 = sub(p2, p0), e12 = sub(p2, p1);
            M.e01x[t] = e01.x; M.e01y[t] = e01.y; M.e01z[t] = e01.z;
            M.e02x[t] = e02.x; M.e02y[t] = e02.y; M.e02z[t] = e02.z;
            M.e12x[t] = e12.x; M.e12y[t] = e12.y; M.e12z[t] = e12.z;
            M.d00[t] = dot(e01, e01);
            M.d00inv[t] = 1. / M.d00[t];
            M.d01[t] = dot(e01, e02);
            M.d11[t] = dot(e02, e02);
            M.d11inv[t] = 1. / M.d11[t];
            M.d22[t] = dot(e12, e12);
            M.d22inv[t] = 1. / M.d22[t];
            M.denom[t] = 1. / (M.d00[t] * M.d11[t] - M.d01[t] * M.d01[t]);
            V3 nn = cross(e01, e02);
            nn = scale(1. / sqrt(dot(nn, nn)), nn);
            M.nx[t] = nn.x; M.ny[t] = nn.y; M.nz[t] = nn.z;
            M.d[t] = -nn.x * X - nn.y * Y - nn.z * Z;
            M.i0[t] = a; M.i1[t] = b; M.i2[t] = c;
            M.cx[t] = (p0.x + p1.x + p2.x) / 3.0;
            M.cy[t] = (p0.y + p1.y + p2.y) / 3.0;
            M.cz[t] = (p0.z + p1.z + p2.z) / 3.0;
            const double P[3][3] = {{p0.x, p1.x, p2.x}, {p0.y, p1.y, p2.y}, {p0.z, p1.z, p2.z}};
            double lo[3], hi[3];
            for (int k = 0; k < 3; k++) {
                lo[k] = P[k][0];
                if (P[k][1] < lo[k]) lo[k] = P[k][1];
                if (P[k][2] < lo[k]) lo[k] = P[k][2];
                hi[k] = P[k][0];
                if (P[k][1] > hi[k]) hi[k] = P[k][1];
                if (P[k][2] > hi[k]) hi[k] = P[k][2];
            }
            M.minx[t] = lo[0]; M.miny[t] = lo[1]; M.minz[t] = lo[2];
            M.maxx[t] = hi[0]; M.maxy[t] = hi[1]; M.maxz[t] = hi[2];
            for (int k = 0; k < 3; k++) {
                if (lo[k] < M.g[k]) M.g[k] = lo[k];
                if (hi[k] > M.g[3 + k]) M.g[3 + k] = hi[k];
            }
        }
    }
    // centroid Morton keys over the mesh AABB (mortonKeyGen, TriangleMesh.cu:4-21)
    const int SCALE = (1 << 10) - 1;
    const double irx = SCALE / (M.g[3] - M.g[0]), iry = SCALE / (M.g[4] - M.g[1]), irz = SCALE / (M.g[5] - M.g[2]);
    M.key.resize(T);
    M.sorted.resize(T);
    for (int q = 0; q < T; q++) {
        M.key[q] = morton((uint32_t)((M.cx[q] - M.g[0]) * irx), (uint32_t)((M.cy[q] - M.g[1]) * iry),
                          (uint32_t)((M.cz[q] - M.g[2]) * irz));
        M.sorted[q] = q;
    }
    lsb_sort(M.key, M.sorted);
}

// median split over the Morton order, children pushed right then left
// (buildBVH, BVH.cu:741-787)
void build_bvh(Bvh& B, const Mesh& M) {
    const int T = M.nTri;
    if (T == 0) return;
    const int maxn = 2 * T - 1;
    for (int k = 0; k < 3; k++) {
        B.lo[k].assign(maxn, 0.);
        B.hi[k].assign(maxn, 0.);
    }
    B.left.assign(maxn, -1);
    B.right.assign(maxn, -1);
    B.tri.assign(maxn, -1);
    struct Task {
        int s, e, node;
    };
    std::vector<Task> st;
    int count = 0;
    st.push_back({0, T, count++});
    const std::vector<double>* lo[3] = {&M.minx, &M.miny, &M.minz};
    const std::vector<double>* hi[3] = {&M.maxx, &M.maxy, &M.maxz};
    while (!st.empty()) {
        Task t = st.back();
        st.pop_back();
        const int f = M.sorted[t.s];
        for (int k = 0; k < 3; k++) {
            double l = (*lo[k])[f], h = (*hi[k])[f];
            for (int q = t.s + 1; q < t.e; q++) {
                const int u = M.sorted[q];
                if ((*lo[k])[u] < l) l = (*lo[k])[u];
                if ((*hi[k])[u] > h) h = (*hi[k])[u];
            }
            B.lo[k][t.node] = l;
            B.hi[k][t.node] = h;
        }
        if (t.e - t.s == 1) {
            B.tri[t.node] = M.sorted[t.s];
            continue;
        }
        const int mid = (t.s + t.e) / 2;
        const int L = count++, R = count++;
        B.left[t.node] = L;
        B.right[t.node] = R;
        st.push_back({mid, t.e, R});
        st.push_back({t.s, mid, L});
    }
    B.nodes = count;
}

// nearest-image x separation with a periodic x
inline double image_dx(const Scene& S, double dx) {
    if (S.per_x) {
        if (dx > S.halfL) dx -= S.L;
        else if (dx < -S.halfL) dx += S.L;
    }
    return dx;
}

// closest feature of triangle t to the centre p within radius^2 rsq
// (dist_triangle cpu_dem.cu:12-205; dist_triangle_neighbor BVH.cu:44-238)
Feature feature_at(const Scene& S, V3 p, int t, double rsq) {
    const Mesh& M = S.mesh;
    Feature res;
    res.n = {0., 0., 0.};
    res.dist = 1.e10;
    res.hit = -2;
    double dist = 0.;
    dist += M.nx[t] * p.x;
    dist += M.ny[t] * p.y;
    dist += M.nz[t] * p.z;
    dist += M.d[t];
    double dsq = dist * dist;
    if (dsq > rsq) return res;
    const int a = M.i0[t], b = M.i1[t], c = M.i2[t];
    const V3 va{M.mx[a], M.my[a], M.mz[a]}, vb{M.mx[b], M.my[b], M.mz[b]}, vc{M.mx[c], M.my[c], M.mz[c]};
    const V3 ap = sub(p, va);
    const double d20 = ap.x * M.e01x[t] + ap.y * M.e01y[t] + ap.z * M.e01z[t];
    const double d21 = ap.x * M.e02x[t] + ap.y * M.e02y[t] + ap.z * M.e02z[t];
    const double v = (M.d11[t] * d20 - M.d01[t] * d21) * M.denom[t];
    const double w = (M.d00[t] * d21 - M.d01[t] * d20) * M.denom[t];
    const double u = 1.0 - v - w;
    if (u > 0. && v > 0. && w > 0.) {
        const double sg = dist < 0 ? -1.0 : 1.0;
        res.n = scale(sg, V3{M.nx[t], M.ny[t], M.nz[t]});
        res.dist = sg * dist;
        res.hit = -1;
        return res;
    }
    V3 q;
    int hit;
    if (v <= 0. && w <= 0.0) {
        q = va;
        hit = a;
    } else if (u <= 0. && w <= 0.0) {
        q = vb;
        hit = b;
    } else if (u <= 0. && v <= 0.0) {
        q = vc;
        hit = c;
    } else if (u <= 0.0) {
        const V3 e{M.e12x[t], M.e12y[t], M.e12z[t]};
        double s = dot(sub(p, vb), e) * M.d22inv[t];
        s = fmax(0., fmin(1.0, s));
        q = add(vb, scale(s, e));
        hit = M.e1[t];
    } else if (v <= 0.0) {
        const V3 e{M.e02x[t], M.e02y[t], M.e02z[t]};
        double s = d21 * M.d11inv[t];
        s = fmax(0., fmin(1.0, s));
        q = add(va, scale(s, e));
        hit = M.e2[t];
    } else {
        const V3 e{M.e01x[t], M.e01y[t], M.e01z[t]};
        double s = d20 * M.d00inv[t];
        s = fmax(0., fmin(1.0, s));
        q = add(va, scale(s, e));
        hit = M.e0[t];
    }
    res.n = sub(p, q);
    dsq = dot(res.n, res.n);
    if (dsq < rsq) {
        res.dist = sqrt(dsq);
        res.n = scale(1. / res.dist, res.n);
    }
    res.hit = hit;
    return res;
}

// ... of particle i, at its x image nearest the triangle's first corner
// with a periodic x (triangles are narrower than a quarter period)
Feature feature(const Scene& S, int i, int t, double rsq) {
    double px = S.x[3 * i];
    if (S.per_x) {
        const double d = px - S.mesh.mx[S.mesh.i0[t]];
        if (d > S.halfL) px -= S.L;
        else if (d < -S.halfL) px += S.L;
    }
    return feature_at(S, V3{px, S.x[3 * i + 1], S.x[3 * i + 2]}, t, rsq);
}

// ------------------------------------------------------------------ cells and lists
inline int cell_of(const Scene& S, double x, int a) {
    if (a == 0 && S.per_x) {
        const int c = (int)floor((x - S.bmin[0]) * S.invx) + 1;
        return c < 1 ? 1 : (c > S.nxp ? S.nxp : c);
    }
    return (int)floor((x - S.bmin[a]) * S.inv) + 1;
}

// canonical CSR: cell-id order, ascending index within a cell (update_pList, BoundingBox.cu:839)
void plist(Scene& S) {
    std::fill(S.pNum.begin(), S.pNum.end(), 0);
    for (int i = 0; i < S.N; i++) {
        if (S.active[i] != 1) continue;
        for (int a = 0; a < 3; a++) S.cellx[3 * i + a] = cell_of(S, S.x[3 * i + a], a);
        S.cellId[i] = (S.size[1] * S.cellx[3 * i + 2] + S.cellx[3 * i + 1]) * S.size[0] + S.cellx[3 * i];
        if (S.cellId[i] < 0 || S.cellId[i] >= S.ncells) {
            fprintf(stderr, "oracle: particle %d outside the cell grid\n", i);
            abort();
        }
        S.pNum[S.cellId[i]] += 1;
    }
    S.pStart[0] = 0;
    for (int c = 1; c < S.ncells; c++) S.pStart[c] = S.pNum[c - 1] + S.pStart[c - 1];
    std::fill(S.cellOff.begin(), S.cellOff.end(), 0);
    for (int i = 0; i < S.N; i++) {
        if (S.active[i] != 1) continue;
        const int c = S.cellId[i];
        S.pList[S.pStart[c] + S.cellOff[c]++] = i;
    }
}

void insertion_sort(int* row, int n) {
    for (int a = 1; a < n; a++) {
        const int t = row[a];
        int b = a;
        while (b > 0 && row[b - 1] > t) {
            row[b] = row[b - 1];
            b--;
        }
        row[b] = t;
    }
}

bool build_lists(Scene& S) {
    plist(S);
    bool ok = true;
    const double skin = S.skin;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < S.N; i++) {
        if (S.active[i] != 1) continue;
        const int cx = S.cellx[3 * i], cy = S.cellx[3 * i + 1], cz = S.cellx[3 * i + 2];
        int nn = 0;
        for (int sx = -1; sx <= 1; sx++)
            for (int sy = -1; sy <= 1; sy++)
                for (int sz = -1; sz <= 1; sz++) {
                    // A particle leaving the box this step is still listed
                    // (main.cu:312-316) and may sit in a ghost cell; the
                    // reference then indexes outside its cell arrays.  Cells
                    // outside the grid hold nobody, so they are skipped.  A
                    // periodic x wraps cells 1..nxp around.
                    int xx = cx + sx;
                    if (S.per_x) {
                        if (xx < 1) xx += S.nxp;
                        else if (xx > S.nxp) xx -= S.nxp;
                    } else if (xx < 0 || xx >= S.size[0]) {
                        continue;
                    }
                    if (cy + sy < 0 || cy + sy >= S.size[1] || cz + sz < 0 || cz + sz >= S.size[2]) continue;
                    const int c = (S.size[1] * (cz + sz) + cy + sy) * S.size[0] + xx;
                    for (int q = S.pStart[c]; q < S.pStart[c] + S.pNum[c]; q++) {
                        const int j = S.pList[q];
                        if (i == j || S.active[j] != 1) continue;
                        const V3 del{image_dx(S, S.x[3 * i] - S.x[3 * j]), S.x[3 * i + 1] - S.x[3 * j + 1],
                                     S.x[3 * i + 2] - S.x[3 * j + 2]};
                        const double dsq = dot(del, del);
                        const double R = S.r[i] + S.r[j] + skin;
                        if (dsq < R * R) {
                            if (nn < K) S.nei[(size_t)i * K + nn] = j;
                            nn++;
                        }
                    }
                }
        if (nn > K) {
            ok = false;
            nn = K;
        }
        S.nnei[i] = nn;
        insertion_sort(&S.nei[(size_t)i * K], nn);
        S.refx[i] = S.x[3 * i];
        S.refy[i] = S.x[3 * i + 1];
        S.refz[i] = S.x[3 * i + 2];
    }
    // wall lists: DFS over the BVH (BVH.cu:576-625)
    if (S.mesh.nTri > 0) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < S.N; i++) {
            if (S.active[i] != 1) continue;
            const double R = S.r[i] + skin;
            const double Rsq = R * R;
            std::vector<int> stack;
            int nn = 0;
            const double py = S.x[3 * i + 1], pz = S.x[3 * i + 2];
            // periodic x: a sphere within R of an x face also queries at its
            // image one period away
            const double x0 = S.x[3 * i];
            const int nimg = S.per_x && (x0 + R > S.bmax[0] || x0 - R < S.bmin[0]) ? 2 : 1;
            for (int img = 0; img < nimg; img++) {
            const double px = img == 0 ? x0 : (x0 + R > S.bmax[0] ? x0 - S.L : x0 + S.L);
            stack.clear();
            stack.push_back(0);
            while (!stack.empty()) {
                const int node = stack.back();
                stack.pop_back();
                double dx = 0.0, dy = 0.0, dz = 0.0;
                if (px < S.bvh.lo[0][node]) dx = S.bvh.lo[0][node] - px;
                else if (px > S.bvh.hi[0][node]) dx = px - S.bvh.hi[0][node];
                if (py < S.bvh.lo[1][node]) dy = S.bvh.lo[1][node] - py;
                else if (py > S.bvh.hi[1][node]) dy = py - S.bvh.hi[1][node];
                if (pz < S.bvh.lo[2][node]) dz = S.bvh.lo[2][node] - pz;
                else if (pz > S.bvh.hi[2][node]) dz = pz - S.bvh.hi[2][node];
                if (!((dx * dx + dy * dy + dz * dz) <= Rsq)) continue;
                if (S.bvh.tri[node] >= 0) {
                    const int t = S.bvh.tri[node];
                    const Feature f = feature_at(S, V3{px, py, pz}, t, Rsq);
                    if (f.dist < S.r[i] + skin) {
                        if (nn < K) S.neiw[(size_t)i * K + nn] = t;
                        nn++;
                    }
                } else {
                    stack.push_back(S.bvh.left[node]);
                    stack.push_back(S.bvh.right[node]);
                }
            }
            }
            if (nn > K) {
                ok = false;
                nn = K;
            }
            S.nneiw[i] = nn;
            insertion_sort(&S.neiw[(size_t)i * K], nn);
        }
    }
    S.rebuilds++;
    return ok;
}

// ------------------------------------------------------------------ forces
// Hertz normal force with Mindlin tangential stiffness for identical
// materials (Tsuji et al. 1992; the damping of the usual DEM form):
//   kn = 4/3 E* sqrt(R* d), Sn = 2 E* sqrt(R* d), kt = 8 G* sqrt(R* d),
//   gamma = -2 sqrt(5/6) beta sqrt(S m*), beta = ln e / sqrt(ln^2 e + pi^2).
// Same operation order as the engine's FP64 kernel.
void hertz(const Scene& S, int i, double Rstar, double mstar, double delMag, double vdn, V3 n, Contact& c) {
    const double damp = S.damp_of(i);
    const double sqrtRd = sqrt(Rstar * delMag);
    const double fel = S.kn_c * sqrtRd * delMag;
    const double gn = damp * sqrt(S.sn_c * sqrtRd * mstar);
    const double fnm = fel - gn * vdn;
    c.fn = {fnm * n.x, fnm * n.y, fnm * n.z};
    c.kt = S.kt_c * sqrtRd;
    c.eta = damp * sqrt(c.kt * mstar);
    c.Rstar = Rstar;
}

Contact normal_pp(Scene& S, int i, int j, V3 n, double delMag) {
    Contact c;
    const V3 del = scale(-delMag, n);
    const V3 vr{S.v[3 * i] - S.v[3 * j], S.v[3 * i + 1] - S.v[3 * j + 1], S.v[3 * i + 2] - S.v[3 * j + 2]};
    const double vdn = dot(vr, n);
    c.vn = scale(vdn, n);
    if (S.model == 1) {
        hertz(S, i, S.r[i] * S.r[j] / (S.r[i] + S.r[j]), 1. / (S.invm[i] + S.invm[j]), delMag, vdn, n, c);
    } else {
        const double meff = 1. / (S.invm[i] + S.invm[j]);
        c.eta = S.eta[i] * sqrt(meff);
        c.kt = S.k[i];
        c.Rstar = 0.;
        c.fn = {-S.k[i] * del.x - c.eta * c.vn.x, -S.k[i] * del.y - c.eta * c.vn.y,
                -S.k[i] * del.z - c.eta * c.vn.z};
    }
    V3 rot{S.r[i] * S.w[3 * i] + S.r[j] * S.w[3 * j], S.r[i] * S.w[3 * i + 1] + S.r[j] * S.w[3 * j + 1],
           S.r[i] * S.w[3 * i + 2] + S.r[j] * S.w[3 * j + 2]};
    rot = cross(rot, n);
    c.vt = add(sub(vr, c.vn), rot);
    S.f[3 * i] += c.fn.x;
    S.f[3 * i + 1] += c.fn.y;
    S.f[3 * i + 2] += c.fn.z;
    c.n = n;
    return c;
}

Contact normal_pw(Scene& S, int i, V3 n, double delMag) {
    Contact c;
    const V3 del = scale(-delMag, n);
    const V3 vr{S.v[3 * i], S.v[3 * i + 1], S.v[3 * i + 2]};
    const double vdn = dot(vr, n);
    c.vn = scale(vdn, n);
    if (S.model == 1) {
        hertz(S, i, S.r[i], 1. / S.invm[i], delMag, vdn, n, c);
    } else {
        c.eta = S.eta[i] * S.sqrtm[i];
        c.kt = S.k[i];
        c.Rstar = 0.;
        c.fn = {-S.k[i] * del.x - c.eta * c.vn.x, -S.k[i] * del.y - c.eta * c.vn.y,
                -S.k[i] * del.z - c.eta * c.vn.z};
    }
    V3 rot{S.r[i] * S.w[3 * i], S.r[i] * S.w[3 * i + 1], S.r[i] * S.w[3 * i + 2]};
    rot = cross(rot, n);
    c.vt = add(sub(vr, c.vn), rot);
    S.f[3 * i] += c.fn.x;
    S.f[3 * i + 1] += c.fn.y;
    S.f[3 * i + 2] += c.fn.z;
    c.n = n;
    return c;
}

// history spring update + Coulomb cap; `key` identifies the partner; `wj`
// is the partner's spin (null for a wall) for the rolling resistance
void tangential(Scene& S, int i, int key, const Contact& c, bool wall, const double* wj) {
    const size_t ci = (size_t)i * K;
    int* id = wall ? S.hwid.data() : S.hid.data();
    int* flag = wall ? S.isCW.data() : S.isC.data();
    int& cnt = wall ? S.ncw[i] : S.nc[i];
    double* hx = wall ? S.hwx.data() : S.hx.data();
    double* hy = wall ? S.hwy.data() : S.hy.data();
    double* hz = wall ? S.hwz.data() : S.hz.data();
    int slot = -1;
    for (int q = 0; q < cnt; q++)
        if (id[ci + q] == key) {
            slot = q;
            break;
        }
    if (slot < 0) {
        slot = cnt;
        id[ci + slot] = key;
        cnt += 1;
        hx[ci + slot] = 0.;
        hy[ci + slot] = 0.;
        hz[ci + slot] = 0.;
    }
    flag[ci + slot] = 1;
    const double dt = S.dt;
    V3 dn{hx[ci + slot] + c.vt.x * dt, hy[ci + slot] + c.vt.y * dt, hz[ci + slot] + c.vt.z * dt};
    dn = sub(dn, scale(dot(dn, c.n), c.n));
    V3 ft = scale(-c.kt, dn);
    const double fnsq = dot(c.fn, c.fn);
    const double ftsq = dot(ft, ft);
    const double mu = S.mu_of(i);
    if (ftsq > (mu * mu) * fnsq) {
        if (ftsq != 0.) {
            const V3 t = scale(1. / (sqrt(ftsq) + 1e-15), ft);
            ft = scale(mu * sqrt(fnsq), t);
            dn = scale(-1. / c.kt, ft);
        } else {
            ft = {0., 0., 0.};
        }
    } else {
        ft.x -= c.eta * c.vt.x;
        ft.y -= c.eta * c.vt.y;
        ft.z -= c.eta * c.vt.z;
    }
    S.f[3 * i] += ft.x;
    S.f[3 * i + 1] += ft.y;
    S.f[3 * i + 2] += ft.z;
    const V3 mm = scale(S.r[i], cross(c.n, ft));
    S.mom[3 * i] += mm.x;
    S.mom[3 * i + 1] += mm.y;
    S.mom[3 * i + 2] += mm.z;
    if (S.model == 1 && S.mu_roll > 0.) {
        // constant rolling resistance opposing the relative spin
        const V3 rel = wj ? V3{S.w[3 * i] - wj[0], S.w[3 * i + 1] - wj[1], S.w[3 * i + 2] - wj[2]}
                          : V3{S.w[3 * i], S.w[3 * i + 1], S.w[3 * i + 2]};
        const double wn = sqrt(dot(rel, rel));
        if (wn > 0.) {
            const double tr = -S.mu_roll * c.Rstar * sqrt(fnsq) / wn;
            S.mom[3 * i] += tr * rel.x;
            S.mom[3 * i + 1] += tr * rel.y;
            S.mom[3 * i + 2] += tr * rel.z;
        }
    }
    hx[ci + slot] = dn.x;
    hy[ci + slot] = dn.y;
    hz[ci + slot] = dn.z;
}

// compaction that leaves the same rows update_history does (cpu_dem.cu:587):
// its swap-with-last loop never re-reads the flag after a swap, so the row is
// cut at the first slot not touched this step, and the cut slots are zeroed.
void compact(Scene& S, int i, bool wall) {
    const size_t ci = (size_t)i * K;
    int* flag = wall ? S.isCW.data() : S.isC.data();
    int& cnt = wall ? S.ncw[i] : S.nc[i];
    int* id = wall ? S.hwid.data() : S.hid.data();
    double* hx = wall ? S.hwx.data() : S.hx.data();
    double* hy = wall ? S.hwy.data() : S.hy.data();
    double* hz = wall ? S.hwz.data() : S.hz.data();
    for (int q = 0; q < cnt; q++) {
        if (flag[ci + q] == 0) {
            const int last = cnt - 1;
            id[ci + q] = id[ci + last];
            hx[ci + q] = hx[ci + last];
            hy[ci + q] = hy[ci + last];
            hz[ci + q] = hz[ci + last];
            hx[ci + last] = 0.;
            hy[ci + last] = 0.;
            hz[ci + last] = 0.;
            cnt -= 1;
            q -= 1;
        }
    }
}

bool step(Scene& S) {
    const int N = S.N;
    std::fill(S.f.begin(), S.f.end(), 0.);
    std::fill(S.mom.begin(), S.mom.end(), 0.);
    std::fill(S.isC.begin(), S.isC.end(), 0);
    std::fill(S.isCW.begin(), S.isCW.end(), 0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
        if (S.active[i] != 1) continue;
        for (int q = 0; q < S.nnei[i]; q++) {
            const int j = S.nei[(size_t)i * K + q];
            if (S.active[j] != 1) continue;
            const V3 del{image_dx(S, S.x[3 * i] - S.x[3 * j]), S.x[3 * i + 1] - S.x[3 * j + 1],
                         S.x[3 * i + 2] - S.x[3 * j + 2]};
            const double dsq = dot(del, del);
            const double R = S.r[i] + S.r[j];
            if (dsq < R * R) {
                const double dist = sqrt(dsq);
                const double delMag = R - dist;
                const V3 n{del.x / dist, del.y / dist, del.z / dist};
                const Contact c = normal_pp(S, i, j, n, delMag);
                tangential(S, i, S.pId[j], c, false, &S.w[3 * j]);
            }
        }
        compact(S, i, false);
    }
    if (S.mesh.nTri > 0) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < N; i++) {
            if (S.active[i] != 1) continue;
            int nvore = 0;
            const size_t ci = (size_t)i * K;
            for (int q = 0; q < S.nneiw[i]; q++) {
                const int t = S.neiw[ci + q];
                const Feature ff = feature(S, i, t, S.rsq[i]);
                if (ff.dist < S.r[i]) {
                    if (ff.hit != -1) {
                        bool dup = false;
                        for (int z = 0; z < nvore; z++)
                            if (S.vore[ci + z] == ff.hit) {
                                dup = true;
                                break;
                            }
                        if (dup) continue;
                        S.vore[ci + nvore++] = ff.hit;
                    }
                    const double delmag = S.r[i] - ff.dist;
                    const Contact c = normal_pw(S, i, ff.n, delmag);
                    tangential(S, i, t, c, true, nullptr);
                }
            }
            compact(S, i, true);
        }
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
        if (S.active[i] != 1) continue;
        for (int a = 0; a < 3; a++) {
            S.a[3 * i + a] = S.f[3 * i + a] * S.invm[i] + S.g[a];
            S.v[3 * i + a] += S.a[3 * i + a] * S.dt;
            S.x[3 * i + a] += S.v[3 * i + a] * S.dt;
        }
        if (S.per_x) {
            if (S.x[3 * i] >= S.bmax[0]) S.x[3 * i] -= S.L;
            else if (S.x[3 * i] < S.bmin[0]) S.x[3 * i] += S.L;
        }
        for (int a = 0; a < 3; a++) {
            S.anga[3 * i + a] = S.mom[3 * i + a] * S.invmoi[i];
            S.w[3 * i + a] += S.anga[3 * i + a] * S.dt;
        }
    }
    bool ok = true;
    bool refresh = false;
    for (int i = 0; i < N && !refresh; i++) {
        if (S.active[i] != 1) continue;
        const V3 del{image_dx(S, S.x[3 * i] - S.refx[i]), S.x[3 * i + 1] - S.refy[i], S.x[3 * i + 2] - S.refz[i]};
        if (dot(del, del) > S.threshSq) refresh = true;
    }
    if (refresh) ok = build_lists(S);
    for (int i = 0; i < N; i++) {
        if (S.active[i] == 0) continue;
        const double X = S.x[3 * i], Y = S.x[3 * i + 1], Z = S.x[3 * i + 2];
        if ((!S.per_x && (X < S.bmin[0] || X > S.bmax[0])) || Y < S.bmin[1] || Y > S.bmax[1] || Z < S.bmin[2] ||
            Z > S.bmax[2])
            S.active[i] = 0;
    }
    S.steps++;
    return ok;
}

}  // namespace

extern "C" {

void* orc_create(int N, const double* x, const double* v, const double* w, const double* r, const double* m,
                 const double* k, const double* eta, double mu, double dt, const double* g, int nTri,
                 const double* tris, const int* files, int nfiles, const double* bmin, const double* bmax,
                 double skin, double thresh, int model, double E, double nu, double e, double mu_roll,
                 int periodic_x) {
    Scene* S = new Scene();
    S->N = N;
    S->dt = dt;
    S->mu = mu;
    S->model = model;
    S->mu_roll = mu_roll;
    if (model == 1) {
        const double Es = E / (2. * (1. - nu * nu));
        const double Gs = E / (4. * (1. + nu) * (2. - nu));
        const double le = log(e);
        const double beta = le / sqrt(le * le + M_PI * M_PI);
        S->kn_c = 4. / 3. * Es;
        S->sn_c = 2. * Es;
        S->kt_c = 8. * Gs;
        S->damp_c = -2. * sqrt(5. / 6.) * beta;
    }
    for (int a = 0; a < 3; a++) S->g[a] = g[a];
    auto z = [&](std::vector<double>& a, size_t n) { a.assign(n, 0.); };
    for (auto* a : {&S->x, &S->v, &S->a, &S->f, &S->w, &S->anga, &S->mom}) z(*a, 3 * (size_t)N);
    for (auto* a : {&S->r, &S->rsq, &S->invr, &S->k, &S->m, &S->sqrtm, &S->invm, &S->moi, &S->invmoi, &S->eta,
                    &S->refx, &S->refy, &S->refz})
        z(*a, N);
    for (auto* a : {&S->hx, &S->hy, &S->hz, &S->hwx, &S->hwy, &S->hwz}) z(*a, (size_t)N * K);
    for (auto* a : {&S->hid, &S->hwid}) a->assign((size_t)N * K, -1);
    for (auto* a : {&S->vore, &S->isC, &S->isCW, &S->nei, &S->neiw}) a->assign((size_t)N * K, 0);
    for (auto* a : {&S->nc, &S->ncw, &S->nnei, &S->nneiw, &S->cellId}) a->assign(N, 0);
    S->cellx.assign(3 * (size_t)N, 0);
    S->active.assign(N, 1);
    S->pId.resize(N);
    double rmax = 0.;
    for (int i = 0; i < N; i++) {
        for (int a = 0; a < 3; a++) {
            S->x[3 * i + a] = x[3 * i + a];
            S->v[3 * i + a] = v ? v[3 * i + a] : 0.;
            S->w[3 * i + a] = w ? w[3 * i + a] : 0.;
        }
        S->r[i] = r[i];
        S->rsq[i] = S->r[i] * S->r[i];
        S->invr[i] = 1. / S->r[i];
        S->k[i] = k[i];
        S->m[i] = m[i];
        S->sqrtm[i] = sqrt(m[i]);
        S->invm[i] = 1. / m[i];
        S->eta[i] = eta[i];
        S->moi[i] = 2. / 5. * S->m[i] * S->rsq[i];
        S->invmoi[i] = 1. / S->moi[i];
        S->pId[i] = i;
        if (rmax < S->r[i]) rmax = S->r[i];
    }
    if (nTri > 0) {
        ingest(S->mesh, tris, nTri, files, nfiles);
        build_bvh(S->bvh, S->mesh);
    }
    for (int a = 0; a < 3; a++) {
        S->bmin[a] = bmin[a];
        S->bmax[a] = bmax[a];
    }
    S->dx = rmax * 4.;
    S->inv = 1. / S->dx;
    S->skin = skin > 0 ? skin : rmax;
    S->thresh = skin > 0 ? thresh : rmax * 0.5;
    S->threshSq = S->thresh * S->thresh;
    for (int a = 0; a < 3; a++) S->size[a] = (int)ceil((S->bmax[a] - S->bmin[a]) / S->dx) + 2;
    if (periodic_x) {
        S->per_x = 1;
        S->L = S->bmax[0] - S->bmin[0];
        S->halfL = 0.5 * S->L;
        S->nxp = (int)floor(S->L / S->dx);
        if (S->nxp < 3) {
            delete S;
            return nullptr;
        }
        S->invx = (double)S->nxp / S->L;
        S->size[0] = S->nxp + 2;
        for (int i = 0; i < N; i++) {
            double& X = S->x[3 * i];
            if (X >= S->bmax[0] || X < S->bmin[0]) {
                X -= S->L * floor((X - S->bmin[0]) / S->L);
                if (X >= S->bmax[0]) X -= S->L;
                if (X < S->bmin[0]) X += S->L;
            }
        }
    }
    S->ncells = S->size[0] * S->size[1] * S->size[2];
    S->pNum.assign(S->ncells, 0);
    S->pStart.assign(S->ncells, 0);
    S->cellOff.assign(S->ncells, 0);
    S->pList.assign(N, 0);
    build_lists(*S);
    S->rebuilds = 0;
    return S;
}

void orc_destroy(void* h) { delete (Scene*)h; }

// Hertz-Mindlin friction and restitution per particle, the damping factor
// -2 sqrt(5/6) beta from each restitution as the engine's
// gdem_set_particle_materials computes it.  Returns -1 for the linear law.
int orc_set_materials(void* h, const double* mu, const double* e) {
    Scene& S = *(Scene*)h;
    if (S.model != 1) return -1;
    S.mu_p.assign(mu, mu + S.N);
    S.damp_p.resize(S.N);
    for (int i = 0; i < S.N; i++) {
        const double le = log(e[i]);
        const double beta = le / sqrt(le * le + M_PI * M_PI);
        S.damp_p[i] = -2. * sqrt(5. / 6.) * beta;
    }
    return 0;
}

int orc_step(void* h, int nsteps) {
    Scene* S = (Scene*)h;
    const long before = S->rebuilds;
    for (int s = 0; s < nsteps; s++)
        if (!step(*S)) return -1;
    return (int)(S->rebuilds - before);
}

int orc_rebuild(void* h) { return build_lists(*(Scene*)h) ? 0 : -1; }

// Copy the named array to `out` and return its length; a name ending in
// "#len" only returns the length (out may be NULL).
long orc_get(void* h, const char* name, void* out) {
    Scene* S = (Scene*)h;
    std::string nm(name);
    bool len_only = false;
    if (nm.size() > 4 && nm.compare(nm.size() - 4, 4, "#len") == 0) {
        nm.resize(nm.size() - 4);
        len_only = true;
    }
    auto D = [&](const std::vector<double>& a) {
        if (!len_only) memcpy(out, a.data(), a.size() * sizeof(double));
        return (long)a.size();
    };
    auto I = [&](const std::vector<int>& a) {
        if (!len_only) memcpy(out, a.data(), a.size() * sizeof(int));
        return (long)a.size();
    };
    if (nm == "x") return D(S->x);
    if (nm == "v") return D(S->v);
    if (nm == "angv") return D(S->w);
    if (nm == "f") return D(S->f);
    if (nm == "mom") return D(S->mom);
    if (nm == "isActive") return I(S->active);
    if (nm == "numCont") return I(S->nc);
    if (nm == "numContWall") return I(S->ncw);
    if (nm == "indHis") return I(S->hid);
    if (nm == "indHisWall") return I(S->hwid);
    if (nm == "deltHisx") return D(S->hx);
    if (nm == "deltHisy") return D(S->hy);
    if (nm == "deltHisz") return D(S->hz);
    if (nm == "deltHisxWall") return D(S->hwx);
    if (nm == "deltHisyWall") return D(S->hwy);
    if (nm == "deltHiszWall") return D(S->hwz);
    if (nm == "numNei") return I(S->nnei);
    if (nm == "neiList") return I(S->nei);
    if (nm == "numNeiWall") return I(S->nneiw);
    if (nm == "neiListWall") return I(S->neiw);
    if (nm == "refx") return D(S->refx);
    if (nm == "refy") return D(S->refy);
    if (nm == "refz") return D(S->refz);
    if (nm == "pNum") return I(S->pNum);
    if (nm == "pStart") return I(S->pStart);
    if (nm == "pList") return I(S->pList);
    if (nm == "cellId") return I(S->cellId);
    if (nm == "cellx") return I(S->cellx);
    const Mesh& M = S->mesh;
    if (nm == "mesh_nx") return D(M.nx);
    if (nm == "mesh_ny") return D(M.ny);
    if (nm == "mesh_nz") return D(M.nz);
    if (nm == "mesh_d") return D(M.d);
    if (nm == "mesh_e01x") return D(M.e01x);
    if (nm == "mesh_e01y") return D(M.e01y);
    if (nm == "mesh_e01z") return D(M.e01z);
    if (nm == "mesh_e02x") return D(M.e02x);
    if (nm == "mesh_e02y") return D(M.e02y);
    if (nm == "mesh_e02z") return D(M.e02z);
    if (nm == "mesh_e12x") return D(M.e12x);
    if (nm == "mesh_e12y") return D(M.e12y);
    if (nm == "mesh_e12z") return D(M.e12z);
    if (nm == "mesh_d00") return D(M.d00);
    if (nm == "mesh_d00inv") return D(M.d00inv);
    if (nm == "mesh_d01") return D(M.d01);
    if (nm == "mesh_d11") return D(M.d11);
    if (nm == "mesh_d11inv") return D(M.d11inv);
    if (nm == "mesh_d22") return D(M.d22);
    if (nm == "mesh_d22inv") return D(M.d22inv);
    if (nm == "mesh_denom") return D(M.denom);
    if (nm == "mesh_minx") return D(M.minx);
    if (nm == "mesh_miny") return D(M.miny);
    if (nm == "mesh_minz") return D(M.minz);
    if (nm == "mesh_maxx") return D(M.maxx);
    if (nm == "mesh_maxy") return D(M.maxy);
    if (nm == "mesh_maxz") return D(M.maxz);
    if (nm == "mesh_cx") return D(M.cx);
    if (nm == "mesh_cy") return D(M.cy);
    if (nm == "mesh_cz") return D(M.cz);
    if (nm == "mesh_mx") return D(M.mx);
    if (nm == "mesh_my") return D(M.my);
    if (nm == "mesh_mz") return D(M.mz);
    if (nm == "mesh_tri_i0") return I(M.i0);
    if (nm == "mesh_tri_i1") return I(M.i1);
    if (nm == "mesh_tri_i2") return I(M.i2);
    if (nm == "mesh_tri_e0") return I(M.e0);
    if (nm == "mesh_tri_e1") return I(M.e1);
    if (nm == "mesh_tri_e2") return I(M.e2);
    if (nm == "mesh_sortedIndex") return I(M.sorted);
    if (nm == "mesh_mortonKey") {
        if (!len_only) memcpy(out, M.key.data(), M.key.size() * sizeof(uint32_t));
        return (long)M.key.size();
    }
    if (nm == "bvh_left") return I(S->bvh.left);
    if (nm == "bvh_right") return I(S->bvh.right);
    if (nm == "bvh_tri") return I(S->bvh.tri);
    if (nm == "bvh_minx") return D(S->bvh.lo[0]);
    if (nm == "bvh_miny") return D(S->bvh.lo[1]);
    if (nm == "bvh_minz") return D(S->bvh.lo[2]);
    if (nm == "bvh_maxx") return D(S->bvh.hi[0]);
    if (nm == "bvh_maxy") return D(S->bvh.hi[1]);
    if (nm == "bvh_maxz") return D(S->bvh.hi[2]);
    return -1;
}

// update_pList_withSort (BoundingBox.cu:664-731): keys of all particles,
// stable sort, reorder of the particle arrays, CSR in cell-id order.
void orc_plist_withsort(void* h, uint32_t* keys_sorted, int* order) {
    Scene& S = *(Scene*)h;
    const int N = S.N;
    std::vector<uint32_t> key(N);
    std::vector<int> idx(N);
    for (int i = 0; i < N; i++) {
        for (int a = 0; a < 3; a++) S.cellx[3 * i + a] = cell_of(S, S.x[3 * i + a], a);
        S.cellId[i] = (S.size[1] * S.cellx[3 * i + 2] + S.cellx[3 * i + 1]) * S.size[0] + S.cellx[3 * i];
        key[i] = morton((uint32_t)S.cellx[3 * i], (uint32_t)S.cellx[3 * i + 1], (uint32_t)S.cellx[3 * i + 2]);
        idx[i] = i;
    }
    lsb_sort(key, idx);
    auto perm_d = [&](std::vector<double>& a, int w) {
        std::vector<double> b(a.size());
        for (int i = 0; i < N; i++)
            for (int c = 0; c < w; c++) b[(size_t)i * w + c] = a[(size_t)idx[i] * w + c];
        a.swap(b);
    };
    auto perm_i = [&](std::vector<int>& a, int w) {
        std::vector<int> b(a.size());
        for (int i = 0; i < N; i++)
            for (int c = 0; c < w; c++) b[(size_t)i * w + c] = a[(size_t)idx[i] * w + c];
        a.swap(b);
    };
    for (auto* a : {&S.x, &S.v, &S.w}) perm_d(*a, 3);
    for (auto* a : {&S.r, &S.rsq, &S.invr, &S.m, &S.sqrtm, &S.invm, &S.moi, &S.invmoi, &S.eta}) perm_d(*a, 1);
    for (auto* a : {&S.hx, &S.hy, &S.hz, &S.hwx, &S.hwy, &S.hwz}) perm_d(*a, K);
    for (auto* a : {&S.hid, &S.hwid, &S.isC, &S.isCW}) perm_i(*a, K);
    for (auto* a : {&S.nc, &S.ncw, &S.cellId, &S.pId, &S.active}) perm_i(*a, 1);
    perm_i(S.cellx, 3);
    std::fill(S.pNum.begin(), S.pNum.end(), 0);
    for (int i = 0; i < N; i++)
        if (S.active[i] == 1) S.pNum[S.cellId[i]] += 1;
    S.pStart[0] = 0;
    for (int c = 1; c < S.ncells; c++) S.pStart[c] = S.pNum[c - 1] + S.pStart[c - 1];
    std::fill(S.cellOff.begin(), S.cellOff.end(), 0);
    for (int i = 0; i < N; i++) {
        if (S.active[i] != 1) continue;
        const int c = S.cellId[i];
        S.pList[S.pStart[c] + S.cellOff[c]++] = i;
    }
    memcpy(keys_sorted, key.data(), sizeof(uint32_t) * N);
    memcpy(order, idx.data(), sizeof(int) * N);
}

void orc_plist(void* h) { plist(*(Scene*)h); }

void orc_radix_sort(int n, const uint32_t* keys, uint32_t* out, int* perm) {
    std::vector<uint32_t> k(keys, keys + n);
    std::vector<int> idx(n);
    for (int i = 0; i < n; i++) idx[i] = i;
    lsb_sort(k, idx);
    memcpy(out, k.data(), sizeof(uint32_t) * n);
    memcpy(perm, idx.data(), sizeof(int) * n);
}

uint32_t orc_morton3d(uint32_t x, uint32_t y, uint32_t z) { return morton(x, y, z); }

void orc_dist_triangle(void* h, int i, int t, double* out4, int* hit) {
    Scene& S = *(Scene*)h;
    const Feature f = feature(S, i, t, S.rsq[i]);
    out4[0] = f.n.x;
    out4[1] = f.n.y;
    out4[2] = f.n.z;
    out4[3] = f.dist;
    *hit = f.dist < 1e9 ? f.hit : -2;
}

void orc_box(void* h, double* d, int* iv) {
    Scene& S = *(Scene*)h;
    d[0] = S.bmin[0]; d[1] = S.bmin[1]; d[2] = S.bmin[2];
    d[3] = S.bmax[0]; d[4] = S.bmax[1]; d[5] = S.bmax[2];
    d[6] = S.dx; d[7] = S.inv; d[8] = S.skin; d[9] = S.thresh; d[10] = S.threshSq;
    iv[0] = S.size[0]; iv[1] = S.size[1]; iv[2] = S.size[2]; iv[3] = S.ncells;
    iv[4] = S.mesh.nTri; iv[5] = S.bvh.nodes; iv[6] = (int)S.mesh.mx.size();
}

long orc_counter(void* h, const char* name) {
    Scene& S = *(Scene*)h;
    if (!strcmp(name, "steps")) return S.steps;
    if (!strcmp(name, "rebuilds")) return S.rebuilds;
    return -1;
}

int orc_threads(void) { return omp_get_max_threads(); }

}  // extern "C"
