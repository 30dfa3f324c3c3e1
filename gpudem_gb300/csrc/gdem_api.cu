// C ABI of the GB300 DEM engine (include/gdem.h): device memory, mesh
// ingestion, import/export in the reference layout, CUDA-graph stepping with
// the rebuild decision taken on the device, and the per-stage entry points.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/gdem.h"
#include "gdem_internal.cuh"

namespace gdem {
void* step_fp64_kernel(int wall_cap);
void launch_stats(const View& v, double* partials, int nblk, cudaStream_t st);
int stats_blocks(int n);
void launch_keys_probe(const View& v, uint32_t* out, cudaStream_t st);
}  // namespace gdem

using namespace gdem;

struct gdem_handle {
    gdem_desc d;
    int n = 0;
    cudaStream_t st = nullptr;
    std::string err;
    // one device arena for the particle arrays, one for the cells, one for the mesh
    char* arena = nullptr;
    char* cell_arena = nullptr;
    char* mesh_arena = nullptr;
    View v;
    Ctl* ctl = nullptr;
    double* stats_partials = nullptr;
    int stats_nblk = 0;
    // mesh (host copies kept for export)
    int ntri = 0;
    std::vector<double> aabb_h;
    uint32_t* tmorton[2] = {nullptr, nullptr};
    int* tidx[2] = {nullptr, nullptr};
    double* aabb_d = nullptr;
    // scene scalars
    bool imported = false;
    double rmax = 0.;
    double cell = 0., skin = 0., thresh = 0.;
    // graphs
    cudaGraphExec_t gK = nullptr, g1 = nullptr;
    int K = 8;
};

namespace {

int fail(gdem_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    return code;
}

#define CK(call)                                                                            \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(h, GDEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

struct Arena {
    size_t off = 0;
    std::vector<std::pair<void**, size_t>> req;
    template <typename T>
    void add(T** p, size_t count) {
        req.push_back({(void**)p, count * sizeof(T)});
    }
    size_t total() const {
        size_t t = 0;
        for (auto& r : req) t += (r.second + 255) & ~size_t(255);
        return t;
    }
    void bind(char* base) {
        size_t o = 0;
        for (auto& r : req) {
            *r.first = base + o;
            o += (r.second + 255) & ~size_t(255);
        }
    }
};

void destroy_graphs(gdem_handle* h) {
    if (h->gK) cudaGraphExecDestroy(h->gK);
    if (h->g1) cudaGraphExecDestroy(h->g1);
    h->gK = h->g1 = nullptr;
}

// K steps, each followed by a conditional node whose body is the list rebuild;
// the step kernel's last block sets the condition from the refresh flag.
int build_graph(gdem_handle* h, int K, cudaGraphExec_t* out) {
    cudaGraph_t g;
    CK(cudaGraphCreate(&g, 0));
    cudaGraphNode_t prev = nullptr;
    const int grid = (h->n + kBlock - 1) / kBlock;
    void* fn = step_fp64_kernel(h->v.wall_cap);
    for (int k = 0; k < K; k++) {
        cudaGraphConditionalHandle hnd;
        CK(cudaGraphConditionalHandleCreate(&hnd, g, 0, cudaGraphCondAssignDefault));
        int use_cond = 1;
        void* args[3] = {(void*)&h->v, (void*)&hnd, (void*)&use_cond};
        cudaKernelNodeParams kp = {};
        kp.func = fn;
        kp.gridDim = dim3(grid);
        kp.blockDim = dim3(kBlock);
        kp.sharedMemBytes = 0;
        kp.kernelParams = args;
        cudaGraphNode_t sn;
        CK(cudaGraphAddKernelNode(&sn, g, prev ? &prev : nullptr, prev ? 1 : 0, &kp));
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = hnd;
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 1;
        cudaGraphNode_t cn;
        CK(cudaGraphAddNode(&cn, g, &sn, nullptr, 1, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        CK(cudaStreamBeginCaptureToGraph(h->st, body, nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal));
        launch_rebuild(h->v, h->st, h->n, /*force=*/1);
        cudaGraph_t captured;
        CK(cudaStreamEndCapture(h->st, &captured));
        prev = cn;
    }
    CK(cudaGraphInstantiate(out, g, 0));
    cudaGraphDestroy(g);
    return GDEM_OK;
}

// current banks and, for every storage slot, the pId living there
int current(gdem_handle* h, Ctl& c, std::vector<int>& pid) {
    CK(cudaStreamSynchronize(h->st));
    CK(cudaMemcpy(&c, h->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
    pid.resize(h->n);
    CK(cudaMemcpy(pid.data(), h->v.P[c.p].pid, sizeof(int) * h->n, cudaMemcpyDeviceToHost));
    return GDEM_OK;
}

template <typename T>
int dl(gdem_handle* h, std::vector<T>& out, const T* src, size_t cnt) {
    out.resize(cnt);
    CK(cudaMemcpy(out.data(), src, sizeof(T) * cnt, cudaMemcpyDeviceToHost));
    return GDEM_OK;
}

}  // namespace

extern "C" {

const char* gdem_last_error(gdem_handle* h) { return h ? h->err.c_str() : "null handle"; }

int gdem_create(const gdem_desc* desc, gdem_handle** out) {
    gdem_handle* h = nullptr;
    if (!desc || !out) return GDEM_ERR_ARG;
    if (desc->n_particles <= 0) return GDEM_ERR_ARG;
    if (desc->precision != GDEM_FP64) return GDEM_ERR_ARG;   // mixed mode: separate kernels
    if (desc->model != GDEM_LINEAR) return GDEM_ERR_ARG;
    h = new gdem_handle();
    h->d = *desc;
    gdem_desc& d = h->d;
    if (d.nei_capacity <= 0) d.nei_capacity = 64;
    if (d.wall_capacity <= 0) d.wall_capacity = 32;
    if (d.hist_capacity <= 0) d.hist_capacity = 32;
    if (d.hist_wall_capacity <= 0) d.hist_wall_capacity = 16;
    if (d.steps_per_graph <= 0) d.steps_per_graph = 8;
    if (d.nei_capacity > 128 || d.wall_capacity > 64 || d.hist_capacity > 64 ||
        d.hist_wall_capacity > 64) {
        delete h;
        return GDEM_ERR_ARG;
    }
    h->K = d.steps_per_graph;
    const int n = d.n_particles;
    h->n = n;
    cudaError_t e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete h;
        return GDEM_ERR_CUDA;
    }
    View& v = h->v;
    memset(&v, 0, sizeof(v));
    v.n = n;
    v.nei_cap = d.nei_capacity;
    v.wall_cap = d.wall_capacity;
    v.hist_cap = d.hist_capacity;
    v.histw_cap = d.hist_wall_capacity;
    v.store_forces = d.store_forces ? 1 : 0;
    v.reorder = d.reorder == 0 ? 0 : 1;
    if (d.reorder < 0) v.reorder = 1;
    v.rs_blocks = rs_blocks_for(n);
    Arena A;
    for (int b = 0; b < 2; b++) {
        SBank& S = v.S[b];
        A.add(&S.x, n); A.add(&S.y, n); A.add(&S.z, n);
        A.add(&S.vx, n); A.add(&S.vy, n); A.add(&S.vz, n);
        A.add(&S.wx, n); A.add(&S.wy, n); A.add(&S.wz, n);
        A.add(&S.active, n);
        PBank& P = v.P[b];
        A.add(&P.r, n); A.add(&P.rsq, n); A.add(&P.invm, n); A.add(&P.sqrtm, n);
        A.add(&P.invmoi, n); A.add(&P.k, n); A.add(&P.eta, n); A.add(&P.pid, n);
        A.add(&P.nc, n); A.add(&P.hid, (size_t)n * v.hist_cap);
        A.add(&P.hx, (size_t)n * v.hist_cap); A.add(&P.hy, (size_t)n * v.hist_cap);
        A.add(&P.hz, (size_t)n * v.hist_cap);
        A.add(&P.ncw, n); A.add(&P.hwid, (size_t)n * v.histw_cap);
        A.add(&P.hwx, (size_t)n * v.histw_cap); A.add(&P.hwy, (size_t)n * v.histw_cap);
        A.add(&P.hwz, (size_t)n * v.histw_cap);
        A.add(&v.keys[b], n);
        A.add(&v.vals[b], n);
    }
    A.add(&v.nei, (size_t)n * v.nei_cap);
    A.add(&v.nnei, n);
    A.add(&v.neiw, (size_t)n * v.wall_cap);
    A.add(&v.nneiw, n);
    A.add(&v.refx, n); A.add(&v.refy, n); A.add(&v.refz, n);
    if (v.store_forces) {
        A.add(&v.fx, n); A.add(&v.fy, n); A.add(&v.fz, n);
        A.add(&v.tx, n); A.add(&v.ty, n); A.add(&v.tz, n);
        A.add(&v.ftmp, (size_t)6 * n);
    }
    A.add(&v.rs_hist, (size_t)256 * v.rs_blocks);
    A.add(&v.rs_tot, 256);
    A.add(&h->ctl, 1);
    h->stats_nblk = stats_blocks(n);
    A.add(&h->stats_partials, (size_t)16 * h->stats_nblk);
    e = cudaMalloc((void**)&h->arena, A.total());
    if (e != cudaSuccess) {
        cudaStreamDestroy(h->st);
        delete h;
        return GDEM_ERR_CUDA;
    }
    A.bind(h->arena);
    v.ctl = h->ctl;
    cudaMemsetAsync(h->arena, 0, A.total(), h->st);
    cudaStreamSynchronize(h->st);
    v.dt = d.dt;
    v.mu = d.mu;
    v.gx = d.g[0];
    v.gy = d.g[1];
    v.gz = d.g[2];
    v.minx = d.box_min[0]; v.miny = d.box_min[1]; v.minz = d.box_min[2];
    v.maxx = d.box_max[0]; v.maxy = d.box_max[1]; v.maxz = d.box_max[2];
    *out = h;
    return GDEM_OK;
}

int gdem_destroy(gdem_handle* h) {
    if (!h) return GDEM_ERR_ARG;
    cudaStreamSynchronize(h->st);
    destroy_graphs(h);
    cudaFree(h->arena);
    cudaFree(h->cell_arena);
    cudaFree(h->mesh_arena);
    cudaStreamDestroy(h->st);
    delete h;
    return GDEM_OK;
}

// ---------------------------------------------------------------- mesh
int gdem_set_mesh(gdem_handle* h, const double* tris, int n_tri, const int* file_tri_counts,
                  int nfiles) {
    if (!h || n_tri < 0 || (n_tri > 0 && !tris)) return fail(h, GDEM_ERR_ARG, "bad mesh arguments");
    cudaStreamSynchronize(h->st);
    destroy_graphs(h);
    cudaFree(h->mesh_arena);
    h->mesh_arena = nullptr;
    h->ntri = n_tri;
    h->v.ntri = n_tri;
    h->v.tri = nullptr;
    h->v.bvh = nullptr;
    h->v.bvh_root = 0;
    if (n_tri == 0) return GDEM_OK;
    std::vector<int> files;
    if (file_tri_counts && nfiles > 0) {
        long tot = 0;
        for (int f = 0; f < nfiles; f++) {
            files.push_back(file_tri_counts[f]);
            tot += file_tri_counts[f];
        }
        if (tot != n_tri) return fail(h, GDEM_ERR_ARG, "file_tri_counts do not sum to n_tri");
    } else {
        files.push_back(n_tri);
    }
    // ---- welding within each file (TriangleMesh.cu:483-533): a vertex takes
    // the index of the first vertex with the same 1e-9-quantised coordinates;
    // indices continue across files; coordinates are those of the first one.
    struct Key {
        long long x, y, z;
        bool operator==(const Key& o) const { return x == o.x && y == o.y && z == o.z; }
    };
    struct KH {
        size_t operator()(const Key& k) const {
            unsigned long long h = 1469598103934665603ULL;
            h ^= (unsigned long long)k.x; h *= 1099511628211ULL;
            h ^= (unsigned long long)k.y; h *= 1099511628211ULL;
            h ^= (unsigned long long)k.z; h *= 1099511628211ULL;
            return (size_t)h;
        }
    };
    const int T = n_tri;
    const int nShift = 3 * T;
    std::vector<double> vx, vy, vz;
    vx.reserve(3 * T); vy.reserve(3 * T); vz.reserve(3 * T);
    std::vector<int> tv(3 * T), te(3 * T);
    std::vector<double> raw3(3 * T);
    std::unordered_map<unsigned long long, int> edges;
    edges.reserve(3 * T);
    int nEdge = 0;
    int t0 = 0;
    for (int f : files) {
        std::unordered_map<Key, int, KH> weld;
        weld.reserve(3 * f);
        for (int t = t0; t < t0 + f; t++) {
            int id[3];
            for (int c = 0; c < 3; c++) {
                const double x = tris[9 * t + 3 * c], y = tris[9 * t + 3 * c + 1],
                             z = tris[9 * t + 3 * c + 2];
                Key k{llround(x / 1e-9), llround(y / 1e-9), llround(z / 1e-9)};
                auto it = weld.find(k);
                if (it == weld.end()) {
                    const int nid = (int)vx.size();
                    weld.emplace(k, nid);
                    vx.push_back(x); vy.push_back(y); vz.push_back(z);
                    id[c] = nid;
                } else {
                    id[c] = it->second;
                }
            }
            raw3[3 * t] = tris[9 * t + 6];
            raw3[3 * t + 1] = tris[9 * t + 7];
            raw3[3 * t + 2] = tris[9 * t + 8];
            // ascending vertex ids (sort3, TriangleMesh.cu:89-103)
            int a = id[0], b = id[1], c = id[2], tmp;
            if (a > b) { tmp = a; a = b; b = tmp; }
            if (b > c) { tmp = b; b = c; c = tmp; }
            if (a > b) { tmp = a; a = b; b = tmp; }
            tv[3 * t] = a; tv[3 * t + 1] = b; tv[3 * t + 2] = c;
            // edges numbered in order of first appearance (get_edge_index, TriangleMesh.cu:73)
            const int pairs[3][2] = {{a, b}, {b, c}, {a, c}};
            for (int q = 0; q < 3; q++) {
                const unsigned long long key =
                    ((unsigned long long)(unsigned)pairs[q][0] << 32) | (unsigned)pairs[q][1];
                auto it = edges.find(key);
                int eid;
                if (it == edges.end()) {
                    eid = nEdge++;
                    edges.emplace(key, eid);
                } else {
                    eid = it->second;
                }
                te[3 * t + q] = eid + nShift;
            }
        }
        t0 += f;
    }
    // ---- triangle AABBs and the mesh AABB, in the loader's comparison order
    h->aabb_h.assign(6 * T, 0.);
    double g[6] = {1e300, 1e300, 1e300, -1e300, -1e300, -1e300};
    for (int t = 0; t < T; t++) {
        const int a = tv[3 * t], b = tv[3 * t + 1], c = tv[3 * t + 2];
        const double* P[3] = {vx.data(), vy.data(), vz.data()};
        for (int k = 0; k < 3; k++) {
            double mn = P[k][a], mx = P[k][a];
            if (P[k][b] < mn) mn = P[k][b];
            if (P[k][c] < mn) mn = P[k][c];
            if (P[k][b] > mx) mx = P[k][b];
            if (P[k][c] > mx) mx = P[k][c];
            h->aabb_h[6 * t + k] = mn;
            h->aabb_h[6 * t + 3 + k] = mx;
        }
        for (int k = 0; k < 3; k++) {
            if (h->aabb_h[6 * t + k] < g[k]) g[k] = h->aabb_h[6 * t + k];
        }
        for (int k = 0; k < 3; k++) {
            if (h->aabb_h[6 * t + 3 + k] > g[3 + k]) g[3 + k] = h->aabb_h[6 * t + 3 + k];
        }
    }
    const int SCALE = (1 << 10) - 1;
    double inv[3];
    for (int k = 0; k < 3; k++) inv[k] = SCALE / (g[3 + k] - g[k]);
    // ---- device side
    const int NV = (int)vx.size();
    Arena M;
    TriRec* rec;
    BNode* nodes;
    double *dvx, *dvy, *dvz, *draw3;
    int *dtv, *dte, *flags;
    M.add(&rec, T);
    M.add(&nodes, 2 * T);
    M.add(&h->aabb_d, 6 * T);
    M.add(&dvx, NV); M.add(&dvy, NV); M.add(&dvz, NV);
    M.add(&draw3, 3 * T);
    M.add(&dtv, 3 * T); M.add(&dte, 3 * T);
    M.add(&flags, T);
    M.add(&h->tmorton[0], T); M.add(&h->tmorton[1], T);
    M.add(&h->tidx[0], T); M.add(&h->tidx[1], T);
    uint32_t *hist, *tot;
    const int nb = rs_blocks_for(T);
    M.add(&hist, (size_t)256 * nb);
    M.add(&tot, 256);
    CK(cudaMalloc((void**)&h->mesh_arena, M.total()));
    M.bind(h->mesh_arena);
    CK(cudaMemcpyAsync(dvx, vx.data(), sizeof(double) * NV, cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(dvy, vy.data(), sizeof(double) * NV, cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(dvz, vz.data(), sizeof(double) * NV, cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(draw3, raw3.data(), sizeof(double) * 3 * T, cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(dtv, tv.data(), sizeof(int) * 3 * T, cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(dte, te.data(), sizeof(int) * 3 * T, cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(h->aabb_d, h->aabb_h.data(), sizeof(double) * 6 * T, cudaMemcpyHostToDevice,
                       h->st));
    launch_tri_precompute(rec, h->aabb_d, h->tmorton[0], h->tidx[0], dvx, dvy, dvz, dtv, dte, draw3,
                          T, g, inv, h->st);
    // stable sort of the centroid keys (radixSortUint32 at TriangleMesh.cu:722)
    radix_sort_pairs(h->tmorton[0], h->tidx[0], h->tmorton[1], h->tidx[1], hist, tot, T, nb, 0, 4,
                     h->st);
    launch_bvh_build(rec, h->aabb_d, nodes, h->tmorton[0], h->tidx[0], flags, T, h->st);
    CK(cudaStreamSynchronize(h->st));
    CK(cudaGetLastError());
    h->v.tri = rec;
    h->v.bvh = nodes;
    h->v.bvh_root = 0;
    if (h->imported) return gdem_rebuild(h);
    return GDEM_OK;
}

int gdem_export_mesh(gdem_handle* h, double* rec, int* irec, double* aabb, uint32_t* morton,
                     int* sorted_index) {
    if (!h) return GDEM_ERR_ARG;
    const int T = h->ntri;
    if (T == 0) return GDEM_OK;
    CK(cudaStreamSynchronize(h->st));
    std::vector<TriRec> R(T);
    CK(cudaMemcpy(R.data(), h->v.tri, sizeof(TriRec) * T, cudaMemcpyDeviceToHost));
    for (int t = 0; t < T; t++) {
        if (rec) memcpy(rec + 29 * (size_t)t, &R[t], 29 * sizeof(double));
        if (irec) memcpy(irec + 6 * (size_t)t, &R[t].i0, 6 * sizeof(int));
    }
    if (aabb) memcpy(aabb, h->aabb_h.data(), sizeof(double) * 6 * T);
    if (morton) CK(cudaMemcpy(morton, h->tmorton[0], sizeof(uint32_t) * T, cudaMemcpyDeviceToHost));
    if (sorted_index) CK(cudaMemcpy(sorted_index, h->tidx[0], sizeof(int) * T, cudaMemcpyDeviceToHost));
    return GDEM_OK;
}

// ---------------------------------------------------------------- particles
int gdem_import_particles(gdem_handle* h, const gdem_particles* p) {
    if (!h || !p || p->n != h->n || !p->x || !p->r || !p->m || !p->k || !p->etaconst)
        return fail(h, GDEM_ERR_ARG, "import: missing arrays or wrong n");
    const int n = h->n;
    CK(cudaStreamSynchronize(h->st));
    destroy_graphs(h);
    View& v = h->v;
    // host staging in engine layout, row = pId
    std::vector<double> x(n), y(n), z(n), vx(n, 0.), vy(n, 0.), vz(n, 0.), wx(n, 0.), wy(n, 0.),
        wz(n, 0.), r(n), rsq(n), invm(n), sqrtm(n), invmoi(n), k(n), eta(n);
    std::vector<int> act(n, 1), pid(n), nc(n, 0), ncw(n, 0);
    const int H = v.hist_cap, HW = v.histw_cap;
    std::vector<int> hid((size_t)n * H, -1), hwid((size_t)n * HW, -1);
    std::vector<double> hx((size_t)n * H, 0.), hy((size_t)n * H, 0.), hz((size_t)n * H, 0.);
    std::vector<double> hwx((size_t)n * HW, 0.), hwy((size_t)n * HW, 0.), hwz((size_t)n * HW, 0.);
    double rmax = 0.;
    for (int i = 0; i < n; i++) {
        x[i] = p->x[3 * i]; y[i] = p->x[3 * i + 1]; z[i] = p->x[3 * i + 2];
        if (p->v) { vx[i] = p->v[3 * i]; vy[i] = p->v[3 * i + 1]; vz[i] = p->v[3 * i + 2]; }
        if (p->angv) { wx[i] = p->angv[3 * i]; wy[i] = p->angv[3 * i + 1]; wz[i] = p->angv[3 * i + 2]; }
        r[i] = p->r[i];
        // derived per-particle constants, ParticleSystem.cu:294-333 operation order
        rsq[i] = r[i] * r[i];
        sqrtm[i] = sqrt(p->m[i]);
        invm[i] = 1. / p->m[i];
        const double moi = 2. / 5. * p->m[i] * rsq[i];
        invmoi[i] = 1. / moi;
        k[i] = p->k[i];
        eta[i] = p->etaconst[i];
        if (p->isActive) act[i] = p->isActive[i];
        pid[i] = i;
        if (rmax < r[i]) rmax = r[i];
        if (p->numCont && p->indHis && p->hist_stride > 0) {
            nc[i] = p->numCont[i];
            if (nc[i] > H) return fail(h, GDEM_ERR_CAPACITY, "import: history longer than hist_capacity");
            for (int s = 0; s < nc[i]; s++) {
                const size_t src = (size_t)i * p->hist_stride + s, dst = (size_t)s * n + i;
                hid[dst] = p->indHis[src];
                hx[dst] = p->deltHisx[src];
                hy[dst] = p->deltHisy[src];
                hz[dst] = p->deltHisz[src];
            }
        }
        if (p->numContWall && p->indHisWall && p->hist_stride > 0) {
            ncw[i] = p->numContWall[i];
            if (ncw[i] > HW)
                return fail(h, GDEM_ERR_CAPACITY, "import: wall history longer than hist_wall_capacity");
            for (int s = 0; s < ncw[i]; s++) {
                const size_t src = (size_t)i * p->hist_stride + s, dst = (size_t)s * n + i;
                hwid[dst] = p->indHisWall[src];
                hwx[dst] = p->deltHisxWall[src];
                hwy[dst] = p->deltHisyWall[src];
                hwz[dst] = p->deltHiszWall[src];
            }
        }
    }
    // ---- grid (initialize_BoundingBox, BoundingBox.cu:370-396)
    h->rmax = rmax;
    h->cell = h->d.cell_size > 0 ? h->d.cell_size : rmax * 4.;
    h->skin = h->d.skin > 0 ? h->d.skin : rmax;
    h->thresh = h->d.refresh_thresh > 0 ? h->d.refresh_thresh : h->skin * 0.5;
    if (2. * rmax + h->skin > h->cell)
        return fail(h, GDEM_ERR_ARG, "cell size smaller than the largest list cutoff 2*r_max+skin");
    v.skin = h->skin;
    v.thresh_sq = h->thresh * h->thresh;
    v.invdx = 1. / h->cell;
    v.invdy = 1. / h->cell;
    v.invdz = 1. / h->cell;
    v.sizex = (int)ceil((v.maxx - v.minx) / h->cell) + 2;
    v.sizey = (int)ceil((v.maxy - v.miny) / h->cell) + 2;
    v.sizez = (int)ceil((v.maxz - v.minz) / h->cell) + 2;
    if (v.sizex > 1024 || v.sizey > 1024 || v.sizez > 1024)
        return fail(h, GDEM_ERR_RANGE, "cell grid exceeds 1024 cells per axis (10-bit Morton keys)");
    v.ncells = v.sizex * v.sizey * v.sizez;
    cudaFree(h->cell_arena);
    h->cell_arena = nullptr;
    Arena Cc;
    Cc.add(&v.cell_start, v.ncells);
    Cc.add(&v.cell_end, v.ncells);
    CK(cudaMalloc((void**)&h->cell_arena, Cc.total()));
    Cc.bind(h->cell_arena);
    // ---- upload into bank 0
    cudaStream_t st = h->st;
    const SBank& S = v.S[0];
    const PBank& P = v.P[0];
#define UP(dst, src, cnt) CK(cudaMemcpyAsync(dst, src.data(), sizeof(src[0]) * (cnt), cudaMemcpyHostToDevice, st))
    UP(S.x, x, n); UP(S.y, y, n); UP(S.z, z, n);
    UP(S.vx, vx, n); UP(S.vy, vy, n); UP(S.vz, vz, n);
    UP(S.wx, wx, n); UP(S.wy, wy, n); UP(S.wz, wz, n);
    UP(S.active, act, n);
    UP(P.r, r, n); UP(P.rsq, rsq, n); UP(P.invm, invm, n); UP(P.sqrtm, sqrtm, n);
    UP(P.invmoi, invmoi, n); UP(P.k, k, n); UP(P.eta, eta, n); UP(P.pid, pid, n);
    UP(P.nc, nc, n); UP(P.hid, hid, (size_t)n * H); UP(P.hx, hx, (size_t)n * H);
    UP(P.hy, hy, (size_t)n * H); UP(P.hz, hz, (size_t)n * H);
    UP(P.ncw, ncw, n); UP(P.hwid, hwid, (size_t)n * HW); UP(P.hwx, hwx, (size_t)n * HW);
    UP(P.hwy, hwy, (size_t)n * HW); UP(P.hwz, hwz, (size_t)n * HW);
#undef UP
    Ctl c0;
    memset(&c0, 0, sizeof(c0));
    CK(cudaMemcpyAsync(h->ctl, &c0, sizeof(Ctl), cudaMemcpyHostToDevice, st));
    if (v.store_forces) {
        CK(cudaMemsetAsync(v.fx, 0, sizeof(double) * n, st));
        CK(cudaMemsetAsync(v.fy, 0, sizeof(double) * n, st));
        CK(cudaMemsetAsync(v.fz, 0, sizeof(double) * n, st));
        CK(cudaMemsetAsync(v.tx, 0, sizeof(double) * n, st));
        CK(cudaMemsetAsync(v.ty, 0, sizeof(double) * n, st));
        CK(cudaMemsetAsync(v.tz, 0, sizeof(double) * n, st));
    }
    CK(cudaStreamSynchronize(st));
    h->imported = true;
    return gdem_rebuild(h);
}

int gdem_rebuild(gdem_handle* h) {
    if (!h || !h->imported) return fail(h, GDEM_ERR_STATE, "rebuild before import");
    launch_finalize_oob(h->v, h->st);
    launch_rebuild(h->v, h->st, h->n, /*force=*/1);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->st));
    unsigned err = 0;
    CK(cudaMemcpy(&err, &h->ctl->error, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (err) return fail(h, GDEM_ERR_DEVICE, "device error word set during rebuild");
    return GDEM_OK;
}

int gdem_step(gdem_handle* h, int nsteps) {
    if (!h || !h->imported) return fail(h, GDEM_ERR_STATE, "step before import");
    if (nsteps < 0) return fail(h, GDEM_ERR_ARG, "negative step count");
    if (!h->gK) {
        int rc = build_graph(h, h->K, &h->gK);
        if (rc) return rc;
        rc = build_graph(h, 1, &h->g1);
        if (rc) return rc;
    }
    const int full = nsteps / h->K, rest = nsteps % h->K;
    for (int q = 0; q < full; q++) CK(cudaGraphLaunch(h->gK, h->st));
    for (int q = 0; q < rest; q++) CK(cudaGraphLaunch(h->g1, h->st));
    return GDEM_OK;
}

int gdem_synchronize(gdem_handle* h) {
    if (!h) return GDEM_ERR_ARG;
    CK(cudaStreamSynchronize(h->st));
    CK(cudaGetLastError());
    unsigned err = 0;
    CK(cudaMemcpy(&err, &h->ctl->error, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (err) return fail(h, GDEM_ERR_DEVICE, "device error word set");
    return GDEM_OK;
}

int gdem_export_particles(gdem_handle* h, gdem_particles* p) {
    if (!h || !p || p->n != h->n) return fail(h, GDEM_ERR_ARG, "export: wrong n");
    if (!h->imported) return fail(h, GDEM_ERR_STATE, "export before import");
    const int n = h->n;
    Ctl c;
    std::vector<int> pid;
    int rc = current(h, c, pid);
    if (rc) return rc;
    const SBank& S = h->v.S[c.s];
    const PBank& P = h->v.P[c.p];
    std::vector<double> a, b, d;
    auto vec3 = [&](double* out, const double* X, const double* Y, const double* Z) -> int {
        int r2 = dl(h, a, X, n) | dl(h, b, Y, n) | dl(h, d, Z, n);
        if (r2) return r2;
        for (int i = 0; i < n; i++) {
            out[3 * pid[i]] = a[i];
            out[3 * pid[i] + 1] = b[i];
            out[3 * pid[i] + 2] = d[i];
        }
        return 0;
    };
    if (p->x && (rc = vec3(p->x, S.x, S.y, S.z))) return rc;
    if (p->v && (rc = vec3(p->v, S.vx, S.vy, S.vz))) return rc;
    if (p->angv && (rc = vec3(p->angv, S.wx, S.wy, S.wz))) return rc;
    if (p->f) {
        if (!h->v.store_forces) return fail(h, GDEM_ERR_STATE, "forces not stored (store_forces=0)");
        if ((rc = vec3(p->f, h->v.fx, h->v.fy, h->v.fz))) return rc;
    }
    if (p->mom) {
        if (!h->v.store_forces) return fail(h, GDEM_ERR_STATE, "forces not stored (store_forces=0)");
        if ((rc = vec3(p->mom, h->v.tx, h->v.ty, h->v.tz))) return rc;
    }
    std::vector<int> iv;
    if (p->isActive) {
        if ((rc = dl(h, iv, S.active, n))) return rc;
        for (int i = 0; i < n; i++) p->isActive[pid[i]] = iv[i] == 1 ? 1 : 0;
    }
    auto scal = [&](double* out, const double* src) -> int {
        int r2 = dl(h, a, src, n);
        if (r2) return r2;
        for (int i = 0; i < n; i++) out[pid[i]] = a[i];
        return 0;
    };
    if (p->r && (rc = scal(p->r, P.r))) return rc;
    if (p->k && (rc = scal(p->k, P.k))) return rc;
    if (p->etaconst && (rc = scal(p->etaconst, P.eta))) return rc;
    if (p->m) {
        if ((rc = dl(h, a, P.invm, n))) return rc;
        for (int i = 0; i < n; i++) p->m[pid[i]] = 1. / a[i];
    }
    const int st = p->hist_stride;
    if (p->numCont && st > 0) {
        const int H = h->v.hist_cap;
        std::vector<int> nc, hid;
        std::vector<double> hx, hy, hz;
        if ((rc = dl(h, nc, P.nc, n)) || (rc = dl(h, hid, P.hid, (size_t)n * H)) ||
            (rc = dl(h, hx, P.hx, (size_t)n * H)) || (rc = dl(h, hy, P.hy, (size_t)n * H)) ||
            (rc = dl(h, hz, P.hz, (size_t)n * H)))
            return rc;
        for (int i = 0; i < n; i++) {
            const int q = pid[i];
            p->numCont[q] = nc[i];
            for (int s = 0; s < nc[i] && s < st; s++) {
                const size_t src = (size_t)s * n + i, dst = (size_t)q * st + s;
                if (p->indHis) p->indHis[dst] = hid[src];
                if (p->deltHisx) p->deltHisx[dst] = hx[src];
                if (p->deltHisy) p->deltHisy[dst] = hy[src];
                if (p->deltHisz) p->deltHisz[dst] = hz[src];
            }
        }
    }
    if (p->numContWall && st > 0) {
        const int H = h->v.histw_cap;
        std::vector<int> nc, hid;
        std::vector<double> hx, hy, hz;
        if ((rc = dl(h, nc, P.ncw, n)) || (rc = dl(h, hid, P.hwid, (size_t)n * H)) ||
            (rc = dl(h, hx, P.hwx, (size_t)n * H)) || (rc = dl(h, hy, P.hwy, (size_t)n * H)) ||
            (rc = dl(h, hz, P.hwz, (size_t)n * H)))
            return rc;
        for (int i = 0; i < n; i++) {
            const int q = pid[i];
            p->numContWall[q] = nc[i];
            for (int s = 0; s < nc[i] && s < st; s++) {
                const size_t src = (size_t)s * n + i, dst = (size_t)q * st + s;
                if (p->indHisWall) p->indHisWall[dst] = hid[src];
                if (p->deltHisxWall) p->deltHisxWall[dst] = hx[src];
                if (p->deltHisyWall) p->deltHisyWall[dst] = hy[src];
                if (p->deltHiszWall) p->deltHiszWall[dst] = hz[src];
            }
        }
    }
    return GDEM_OK;
}

int gdem_export_lists(gdem_handle* h, int stride, int* numNei, int* neiList, int* numNeiWall,
                      int* neiListWall) {
    if (!h || stride <= 0) return fail(h, GDEM_ERR_ARG, "export_lists: bad stride");
    if (!h->imported) return fail(h, GDEM_ERR_STATE, "export before import");
    const int n = h->n;
    Ctl c;
    std::vector<int> pid;
    int rc = current(h, c, pid);
    if (rc) return rc;
    std::vector<int> cnt, rows;
    if (numNei || neiList) {
        if ((rc = dl(h, cnt, (const int*)h->v.nnei, n)) ||
            (rc = dl(h, rows, (const int*)h->v.nei, (size_t)n * h->v.nei_cap)))
            return rc;
        for (int i = 0; i < n; i++) {
            const int q = pid[i];
            if (numNei) numNei[q] = cnt[i];
            if (neiList)
                for (int k = 0; k < cnt[i] && k < stride; k++)
                    neiList[(size_t)q * stride + k] = pid[rows[(size_t)k * n + i]];
        }
    }
    if (numNeiWall || neiListWall) {
        if ((rc = dl(h, cnt, (const int*)h->v.nneiw, n)) ||
            (rc = dl(h, rows, (const int*)h->v.neiw, (size_t)n * h->v.wall_cap)))
            return rc;
        for (int i = 0; i < n; i++) {
            const int q = pid[i];
            if (numNeiWall) numNeiWall[q] = cnt[i];
            if (neiListWall)
                for (int k = 0; k < cnt[i] && k < stride; k++)
                    neiListWall[(size_t)q * stride + k] = rows[(size_t)k * n + i];
        }
    }
    return GDEM_OK;
}

int gdem_morton_keys(gdem_handle* h, uint32_t* keys) {
    if (!h || !keys) return fail(h, GDEM_ERR_ARG, "morton_keys: null");
    if (!h->imported) return fail(h, GDEM_ERR_STATE, "keys before import");
    const int n = h->n;
    launch_keys_probe(h->v, h->v.keys[1], h->st);
    CK(cudaGetLastError());
    Ctl c;
    std::vector<int> pid;
    int rc = current(h, c, pid);
    if (rc) return rc;
    std::vector<uint32_t> k;
    if ((rc = dl(h, k, (const uint32_t*)h->v.keys[1], n))) return rc;
    for (int i = 0; i < n; i++) keys[pid[i]] = k[i];
    return GDEM_OK;
}

int gdem_export_cells(gdem_handle* h, uint32_t* keys_sorted, int* order, int* pNum, int* pStart,
                      int* pList, int* n_cells) {
    if (!h) return GDEM_ERR_ARG;
    if (!h->imported) return fail(h, GDEM_ERR_STATE, "cells before import");
    const int n = h->n;
    if (n_cells) *n_cells = h->v.ncells;
    if (!keys_sorted && !order && !pNum && !pStart && !pList) return GDEM_OK;
    Ctl c;
    std::vector<int> pid;
    int rc = current(h, c, pid);
    if (rc) return rc;
    std::vector<uint32_t> k;
    std::vector<int> vals, cs, ce;
    if ((rc = dl(h, k, (const uint32_t*)h->v.keys[0], n)) ||
        (rc = dl(h, vals, (const int*)h->v.vals[0], n)) ||
        (rc = dl(h, cs, (const int*)h->v.cell_start, h->v.ncells)) ||
        (rc = dl(h, ce, (const int*)h->v.cell_end, h->v.ncells)))
        return rc;
    if (keys_sorted) memcpy(keys_sorted, k.data(), sizeof(uint32_t) * n);
    // storage index at each sorted position
    std::vector<int> at(n);
    for (int q = 0; q < n; q++) at[q] = h->v.reorder ? q : vals[q];
    if (order)
        for (int q = 0; q < n; q++) order[q] = pid[at[q]];
    int run = 0;
    for (int cc = 0; cc < h->v.ncells; cc++) {
        const int cnt = ce[cc] - cs[cc];
        if (pNum) pNum[cc] = cnt;
        if (pStart) pStart[cc] = run;
        if (pList)
            for (int t = 0; t < cnt; t++) pList[run + t] = at[cs[cc] + t];
        run += cnt;
    }
    return GDEM_OK;
}

int gdem_sort_keys(const uint32_t* keys, int n, uint32_t* keys_sorted, int* perm) {
    if (n < 0 || (n > 0 && (!keys || !keys_sorted || !perm))) return GDEM_ERR_ARG;
    if (n == 0) return GDEM_OK;
    gdem_handle* h = nullptr;
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const int nb = rs_blocks_for(n);
    Arena A;
    uint32_t *k0, *k1, *hist, *tot;
    int *v0, *v1;
    A.add(&k0, n); A.add(&k1, n); A.add(&v0, n); A.add(&v1, n);
    A.add(&hist, (size_t)256 * nb); A.add(&tot, 256);
    char* base;
    CK(cudaMalloc((void**)&base, A.total()));
    A.bind(base);
    std::vector<int> iota(n);
    for (int i = 0; i < n; i++) iota[i] = i;
    cudaMemcpyAsync(k0, keys, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(v0, iota.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
    radix_sort_pairs(k0, v0, k1, v1, hist, tot, n, nb, 0, 4, st);
    cudaMemcpyAsync(keys_sorted, k0, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(perm, v0, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(base);
    cudaStreamDestroy(st);
    return e == cudaSuccess ? GDEM_OK : GDEM_ERR_CUDA;
}

int gdem_dist_triangle(gdem_handle* h, const double* pos, const double* r, const int* tri, int m,
                       double* out4, int* hitAt) {
    if (!h || m < 0) return GDEM_ERR_ARG;
    if (m == 0) return GDEM_OK;
    if (h->ntri == 0) return fail(h, GDEM_ERR_STATE, "no mesh");
    for (int q = 0; q < m; q++)
        if (tri[q] < 0 || tri[q] >= h->ntri) return fail(h, GDEM_ERR_ARG, "triangle index out of range");
    Arena A;
    double *dp, *dr, *dout;
    int *dt, *dh;
    A.add(&dp, 3 * (size_t)m); A.add(&dr, m); A.add(&dt, m); A.add(&dout, 4 * (size_t)m); A.add(&dh, m);
    char* base;
    CK(cudaMalloc((void**)&base, A.total()));
    A.bind(base);
    cudaMemcpyAsync(dp, pos, sizeof(double) * 3 * m, cudaMemcpyHostToDevice, h->st);
    cudaMemcpyAsync(dr, r, sizeof(double) * m, cudaMemcpyHostToDevice, h->st);
    cudaMemcpyAsync(dt, tri, sizeof(int) * m, cudaMemcpyHostToDevice, h->st);
    launch_dist_triangle(h->v.tri, dp, dr, dt, m, dout, dh, h->st);
    cudaMemcpyAsync(out4, dout, sizeof(double) * 4 * m, cudaMemcpyDeviceToHost, h->st);
    cudaMemcpyAsync(hitAt, dh, sizeof(int) * m, cudaMemcpyDeviceToHost, h->st);
    cudaError_t e = cudaStreamSynchronize(h->st);
    cudaFree(base);
    if (e != cudaSuccess) return fail(h, GDEM_ERR_CUDA, cudaGetErrorString(e));
    return GDEM_OK;
}

int gdem_stats_get(gdem_handle* h, gdem_stats* s) {
    if (!h || !s) return GDEM_ERR_ARG;
    if (!h->imported) return fail(h, GDEM_ERR_STATE, "stats before import");
    launch_stats(h->v, h->stats_partials, h->stats_nblk, h->st);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->st));
    std::vector<double> part((size_t)16 * h->stats_nblk);
    CK(cudaMemcpy(part.data(), h->stats_partials, sizeof(double) * part.size(), cudaMemcpyDeviceToHost));
    Ctl c;
    CK(cudaMemcpy(&c, h->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
    // partial layout per block: 0 n_active 1 n_nei 2 n_wall 3 n_cont 4 n_wcont 5 KE 6 vol
    // 7..9 min xyz 10..12 max xyz 13 max overlap
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, mo = 0.;
    for (int b = 0; b < h->stats_nblk; b++) {
        const double* q = &part[(size_t)16 * b];
        for (int k = 0; k < 7; k++) acc[k] += q[k];
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], q[7 + k]);
            hi[k] = std::max(hi[k], q[10 + k]);
        }
        mo = std::max(mo, q[13]);
    }
    memset(s, 0, sizeof(*s));
    s->steps = (long long)c.steps;
    s->rebuilds = (long long)c.rebuilds;
    s->n_active = (long long)acc[0];
    s->n_nei = (long long)acc[1];
    s->n_wall = (long long)acc[2];
    s->n_contacts = (long long)acc[3];
    s->n_wall_contacts = (long long)acc[4];
    s->kinetic_energy = acc[5];
    s->coordination = acc[0] > 0 ? acc[3] / acc[0] : 0.;
    const double vb = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]);
    s->packing_fraction = (acc[0] > 0 && vb > 0) ? acc[6] / vb : 0.;
    s->max_overlap = mo;
    s->error_word = c.error;
    s->max_nei = c.max_nei;
    s->max_wall = c.max_wall;
    return GDEM_OK;
}

int gdem_get_stream(gdem_handle* h, void** stream) {
    if (!h || !stream) return GDEM_ERR_ARG;
    *stream = (void*)h->st;
    return GDEM_OK;
}

int gdem_profile_step(gdem_handle* h, int iters, float* avg_ms) {
    if (!h || iters <= 0 || !avg_ms) return GDEM_ERR_ARG;
    if (!h->imported) return fail(h, GDEM_ERR_STATE, "profile before import");
    std::vector<cudaEvent_t> ev(2 * iters);
    for (auto& e : ev) CK(cudaEventCreate(&e));
    for (int q = 0; q < iters; q++) {
        CK(cudaEventRecord(ev[2 * q], h->st));
        launch_step_fp64(h->v, h->st, 0, 0);
        CK(cudaEventRecord(ev[2 * q + 1], h->st));
        launch_rebuild(h->v, h->st, h->n, /*force=*/0);
    }
    CK(cudaStreamSynchronize(h->st));
    CK(cudaGetLastError());
    double tot = 0.;
    for (int q = 0; q < iters; q++) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ev[2 * q], ev[2 * q + 1]));
        tot += ms;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    *avg_ms = (float)(tot / iters);
    return GDEM_OK;
}

}  // extern "C"
