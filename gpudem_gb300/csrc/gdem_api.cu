// C ABI of the GB300 DEM engine (include/gdem.h): device memory, mesh
// ingestion, import/export in the reference layout, CUDA-graph stepping with
// the rebuild decision taken on the device, and the per-stage entry points.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "../../include/gdem.h"
#include "gdem_internal.cuh"

namespace gdem {
template <class T>
void launch_gather_positions(const View<T>& v, double* out, cudaStream_t st);
}

using namespace gdem;

namespace {

struct Arena {
    std::vector<std::pair<void**, size_t>> req;
    template <typename X>
    void add(X** p, size_t count) {
        req.push_back({(void**)p, count * sizeof(X)});
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

// A host array without value-initialisation (no zero fill before the
// caller writes every element).
template <class X>
struct HostBuf {
    std::unique_ptr<X[]> p;
    explicit HostBuf(size_t count) : p(count ? new X[count] : nullptr) {}
    X* data() { return p.get(); }
    X& operator[](size_t i) { return p[i]; }
    const X& operator[](size_t i) const { return p[i]; }
};

// f(lo, hi) over [0, n) in contiguous chunks, one host thread each (one
// thread for small n); f must not throw.
template <class F>
static void host_parallel_for(int n, F f) {
    unsigned nt = std::thread::hardware_concurrency();
    nt = nt == 0 ? 1u : (nt > 32u ? 32u : nt);
    if (n < (1 << 16)) nt = 1;
    if (nt == 1) {
        f(0, n);
        return;
    }
    const int chunk = (int)((n + nt - 1) / nt);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; t++) {
        const int lo = (int)t * chunk, hi = lo + chunk < n ? lo + chunk : n;
        if (lo >= hi) break;
        th.emplace_back(f, lo, hi);
    }
    for (auto& x : th) x.join();
}

struct MeshData {
    int ntri = 0;
    char* arena = nullptr;
    TriRec* rec = nullptr;
    double* aabb_d = nullptr;
    uint32_t* morton[2] = {nullptr, nullptr};
    int* idx[2] = {nullptr, nullptr};
    uint32_t *hist = nullptr, *tot = nullptr;  // key-sort scratch
    SegBox* seg = nullptr;                     // mesh tree boxes, level by level
    SegBoxF* segf = nullptr;                   // their FP32 copies (mixed-precision list build)
    unsigned* done = nullptr;                  // last-CTA counter of the tree build
    double gmin[3] = {0., 0., 0.}, ginv[3] = {0., 0., 0.};
    double max_diag = 0.;                      // largest triangle bounding-box diagonal
    std::vector<double> aabb_h;
};

// Rebuild the mesh tree of a mesh already set: centroid keys, their stable
// sort, the boxes of every level (the set-up's own steps).
static void launch_bvh_rebuild(const MeshData& M, cudaStream_t st) {
    if (M.ntri <= 0) return;
    launch_tri_keys(M.rec, M.morton[0], M.idx[0], M.ntri, M.gmin, M.ginv, st);
    radix_sort_pairs(M.morton[0], M.idx[0], M.morton[1], M.idx[1], M.hist, M.tot, M.ntri, rs_blocks_for(M.ntri), 0,
                     4, st);
    launch_bvh_build(M.aabb_d, M.idx[0], M.seg, M.segf, M.done, M.ntri, st);
}

// Snapshot file: this header, then per particle in pId order the state
// arrays of the precision (mixed: posh, posl, vel, vell, rot, rotl; FP64: pos,
// vel, rot; 16 or 32 bytes each) and the material record, then the particle
// history (n counts, the live keys, their spring terms) and the wall history
// in the same form.
struct SnapHeader {
    char magic[8];
    int version, n, precision, model, hist_cap, histw_cap, per_particle_mat, rsize;
    unsigned long long steps;
    unsigned error, pad;
};

// Structure of a snapshot file, read without touching a device: the header,
// the exact length, history counts within the stored capacities, and every
// history key an index of this state (partner particles in [0, n), triangles
// in [0, n_tri)).  A snapshot that fails is refused before any upload.
static int check_snapshot_file(const char* path, int n_tri, SnapHeader* out, std::string& msg) {
    FILE* fp = fopen(path, "rb");
    if (!fp) {
        msg = std::string("snapshot: cannot open ") + path;
        return GDEM_ERR_ARG;
    }
    SnapHeader hd;
    bool ok = fread(&hd, 1, sizeof(hd), fp) == sizeof(hd);
    auto bad = [&](const char* why) {
        fclose(fp);
        msg = std::string("snapshot: ") + why;
        return GDEM_ERR_ARG;
    };
    if (!ok || memcmp(hd.magic, "GDEMSNAP", 8) != 0 || hd.version != 1) return bad("not a snapshot file");
    const bool mixed = hd.precision == GDEM_MIXED;
    if (hd.n <= 0 || (hd.precision != GDEM_FP64 && !mixed) || hd.rsize != (mixed ? 4 : 8) || hd.hist_cap < 0 ||
        hd.histw_cap < 0 || hd.hist_cap > 64 || hd.histw_cap > 64)
        return bad("header out of range");
    const size_t n = (size_t)hd.n;
    const int nterms = mixed ? 6 : 3;
    const long state = (long)(n * (mixed ? 7 * 16 : 4 * 32));
    if (fseek(fp, state, SEEK_CUR) != 0) return bad("truncated");
    for (int part = 0; part < 2; part++) {
        const int cap = part == 0 ? hd.hist_cap : hd.histw_cap;
        const long long id_end = part == 0 ? hd.n : n_tri;
        std::vector<int> cnt(n);
        if (fread(cnt.data(), sizeof(int), n, fp) != n) return bad("truncated");
        size_t tot = 0;
        for (size_t q = 0; q < n; q++) {
            if (cnt[q] < 0 || cnt[q] > cap) return bad("a history longer than its capacity");
            tot += (size_t)cnt[q];
        }
        std::vector<int> id(tot);
        if (tot && fread(id.data(), sizeof(int), tot, fp) != tot) return bad("truncated");
        for (size_t e = 0; e < tot; e++)
            if (id[e] < 0 || id[e] >= id_end)
                return bad(part == 0 ? "a history partner outside [0, n)" : "a wall history triangle outside the mesh");
        if (fseek(fp, (long)(tot * nterms * hd.rsize), SEEK_CUR) != 0) return bad("truncated");
    }
    const long here = ftell(fp);
    fseek(fp, 0, SEEK_END);
    const long end = ftell(fp);
    if (here != end) return bad("truncated, or trailing bytes");
    fclose(fp);
    if (out) *out = hd;
    return GDEM_OK;
}

// Everything that depends on the precision mode.
struct EngineBase {
    virtual ~EngineBase() {}
    virtual int import_(const gdem_particles* p) = 0;
    virtual int rebuild() = 0;
    virtual int step(int nsteps) = 0;
    virtual int export_(gdem_particles* p) = 0;
    virtual int export_positions(double* x) = 0;
    virtual int lists(int stride, int* nn, int* nl, int* nw, int* wl) = 0;
    virtual int keys(uint32_t* k) = 0;
    virtual int cells(uint32_t* ks, int* order, int* pNum, int* pStart, int* pList, int* ncell) = 0;
    virtual int stats(gdem_stats* s) = 0;
    virtual int profile(int iters, float* ms) = 0;
    virtual int set_materials(const double* mu, const double* restitution) = 0;
    virtual void set_mesh(const MeshData& m) = 0;
    virtual unsigned error_word() = 0;
    virtual int frame_async(const char* dir, int step, double length_factor) = 0;
    virtual int export_positions_async(double* x) = 0;
    virtual int sync_copies() = 0;
    virtual int frames_flush() = 0;
    virtual int save_snapshot(const char* path) = 0;
    virtual int init_particles(const gdem_inlet* in) = 0;
    virtual int load_snapshot(const char* path) = 0;
    std::string err;
    cudaStream_t st = nullptr;
    bool imported = false;
};

int failv(std::string& e, int code, const std::string& msg) {
    e = msg;
    return code;
}

#define CKE(call)                                                                                \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess)                                                                   \
            return failv(err, GDEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
struct Impl : EngineBase {
    using R = typename T::real;
    using V4 = typename T::v4;
    gdem_desc d;
    int n;
    View<T> v;
    char* arena = nullptr;
    char* cell_arena = nullptr;
    double* stats_partials = nullptr;
    int stats_nblk = 0;
    double* gather = nullptr;  // [3n] pId-ordered positions for fast exports
    cudaGraphExec_t gK = nullptr, g1 = nullptr;
    int K = 8;
    bool use_graphs = true;

    ~Impl() override {
        frames_shutdown();
        if (copy_st) cudaStreamSynchronize(copy_st);
        for (int k = 0; k < 2; k++) {
            cudaFree(pgather[k]);
            if (pready[k]) cudaEventDestroy(pready[k]);
            if (pcopied[k]) cudaEventDestroy(pcopied[k]);
        }
        if (copy_st) cudaStreamDestroy(copy_st);
        if (st) cudaStreamSynchronize(st);
        destroy_graphs();
        cudaFree(arena);
        cudaFree(cell_arena);
        cudaFree(trif);
        if (st) cudaStreamDestroy(st);
    }

    void destroy_graphs() {
        if (gK) cudaGraphExecDestroy(gK);
        if (g1) cudaGraphExecDestroy(g1);
        gK = g1 = nullptr;
    }

    int create(const gdem_desc& desc) {
        d = desc;
        n = d.n_particles;
        K = d.steps_per_graph;
        const char* env = getenv("GDEM_GRAPHS");
        use_graphs = !(env && env[0] == '0');
        CKE(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        memset(&v, 0, sizeof(v));
        v.n = n;
        v.nei_cap = d.nei_capacity;
        v.wall_cap = d.wall_capacity;
        v.hist_cap = d.hist_capacity;
        v.histw_cap = d.hist_wall_capacity;
        v.store_forces = d.store_forces ? 1 : 0;
        v.kernel_variant = d.mixed_kernel >= 0 && d.mixed_kernel <= 3 ? d.mixed_kernel : 0;
        v.occupancy = d.occupancy > 0 ? d.occupancy : 0;
        // failure-detection tests only: fewer tries for the step kernels'
        // pipeline waits, so that a wait gives up and reports GDEM_EW_TIMEOUT
        v.wait_tries = kSpinLimit;
        if (const char* wt = getenv("GDEM_TEST_WAIT_TRIES")) v.wait_tries = (unsigned)strtoul(wt, nullptr, 10);
        v.reorder = d.reorder == 0 ? 0 : 1;
        v.rs_blocks = rs_blocks_for(n);
        const size_t H = (size_t)n * v.hist_cap, HW = (size_t)n * v.histw_cap;
        Arena A;
        for (int b = 0; b < 2; b++) {
            SBank<T>& S = v.S[b];
            if (!T::mixed) A.add(&S.pos, n);
            A.add(&S.vel, n);
            A.add(&S.rot, n);
            if (T::mixed) {
                A.add(&S.posh, n);
                A.add(&S.posl, n);
                A.add(&S.vell, n);
                A.add(&S.rotl, n);
            }
            PBank<T>& P = v.P[b];
            A.add(&P.mat, n);
            A.add(&P.pid, n);
            A.add(&P.nc, n);
            A.add(&P.hid, H);
            A.add(&P.hx, H); A.add(&P.hy, H); A.add(&P.hz, H);
            if (T::mixed) { A.add(&P.cx, H); A.add(&P.cy, H); A.add(&P.cz, H); }
            A.add(&P.ncw, n);
            A.add(&P.hwid, HW);
            A.add(&P.hwx, HW); A.add(&P.hwy, HW); A.add(&P.hwz, HW);
            if (T::mixed) { A.add(&P.cwx, HW); A.add(&P.cwy, HW); A.add(&P.cwz, HW); }
            A.add(&v.keys[b], n);
            A.add(&v.vals[b], n);
        }
        A.add(&v.nei, (size_t)n * v.nei_cap);
        A.add(&v.nnei, n);
        A.add(&v.neiw, (size_t)n * v.wall_cap);
        A.add(&v.nneiw, n);
        if (T::mixed) {
            A.add(&v.refh, n);
            if (d.inner_skin >= 0.) {
                A.add(&v.inn, (size_t)n * v.nei_cap);
                A.add(&v.ninn, n);
                A.add(&v.innw, (size_t)n * v.wall_cap);
                A.add(&v.ninnw, n);
                A.add(&v.refi, n);
            }
        } else {
            A.add(&v.ref, n);
            A.add(&v.posf, n);
        }
        if (v.store_forces) {
            A.add(&v.fx, n); A.add(&v.fy, n); A.add(&v.fz, n);
            A.add(&v.tx, n); A.add(&v.ty, n); A.add(&v.tz, n);
            A.add(&v.ftmp, (size_t)6 * n);
        }
        if (T::mixed) A.add(&v.inv, n);
        A.add(&v.where, n);
        // cell wall-candidate lists: a count and a base per cell start, and
        // the shared buffer (4 entries per particle; a cell that finds it
        // full falls back to the per-particle tree traversal)
        v.cw_cap = 4 * n + 1024;
        A.add(&v.cw_cnt, n);
        A.add(&v.cw_base, n);
        A.add(&v.cw_list, (size_t)v.cw_cap);
        A.add(&v.cell_list, n);
        A.add(&v.cell_bc, (size_t)(n + kBlock - 1) / kBlock + 1);
        A.add(&v.rs_hist, (size_t)256 * v.rs_blocks);
        A.add(&v.rs_tot, 256);
        A.add(&v.ctl, 1);
        stats_nblk = stats_blocks(n);
        A.add(&stats_partials, (size_t)16 * stats_nblk);
        A.add(&gather, (size_t)3 * n);
        CKE(cudaMalloc((void**)&arena, A.total()));
        A.bind(arena);
        CKE(cudaMemsetAsync(arena, 0, A.total(), st));
        CKE(cudaStreamSynchronize(st));
        v.dt = d.dt;
        v.gx = d.g[0];
        v.gy = d.g[1];
        v.gz = d.g[2];
        v.minx = d.box_min[0]; v.miny = d.box_min[1]; v.minz = d.box_min[2];
        v.maxx = d.box_max[0]; v.maxy = d.box_max[1]; v.maxz = d.box_max[2];
        v.per_x = d.periodic_x ? 1 : 0;
        if (v.per_x) {
            v.Lx = v.maxx - v.minx;
            if (!(v.Lx > 0.)) return GDEM_ERR_ARG;
            v.halfLx = 0.5 * v.Lx;
            v.Lxh = (float)v.Lx;
            v.Lxl = (float)(v.Lx - (double)v.Lxh);
            v.halfLxf = (float)v.halfLx;
            // a pair hi + lo below minx (at or above maxx) has hi <= minx
            // (>= maxx) to within half an ulp of hi: test two ulps inside
            float lo = (float)v.minx, hi = (float)v.maxx;
            for (int k = 0; k < 2; k++) {
                lo = nextafterf(lo, INFINITY);
                hi = nextafterf(hi, -INFINITY);
            }
            v.perf[0] = lo;
            v.perf[1] = hi;
        }
        float xmax = 0.f;
        for (int k = 0; k < 3; k++) {
            v.boxf[k] = nextafterf((float)d.box_min[k], -INFINITY);
            v.boxf[3 + k] = nextafterf((float)d.box_max[k], INFINITY);
            xmax = fmaxf(xmax, fmaxf(fabsf(v.boxf[k]), fabsf(v.boxf[3 + k])));
        }
        // a particle still listed while leaving the box lies within twice the
        // largest box coordinate; 8 ulps there bound the FP32 distance error
        v.nb_delta = 8.f * (nextafterf(2.f * xmax, INFINITY) - 2.f * xmax);
        v.dtf = (float)d.dt;
        v.gxf = (float)d.g[0];
        v.gyf = (float)d.g[1];
        v.gzf = (float)d.g[2];
        Material& m = v.mat;
        m.model = d.model;
        m.mu = d.mu;
        m.mu_roll = d.rolling_friction;
        if (d.model == GDEM_HERTZ_MINDLIN) {
            const double E = d.youngs_modulus, nu = d.poisson_ratio, e = d.restitution;
            const double Es = E / (2. * (1. - nu * nu));
            const double Gs = E / (4. * (1. + nu) * (2. - nu));
            const double le = log(e);
            const double beta = le / sqrt(le * le + M_PI * M_PI);
            m.kn_c = 4. / 3. * Es;
            m.sn_c = 2. * Es;
            m.kt_c = 8. * Gs;
            m.damp_c = -2. * sqrt(5. / 6.) * beta;
        }
        v.muf = (float)m.mu;
        v.kn_cf = (float)m.kn_c;
        v.sn_cf = (float)m.sn_c;
        v.kt_cf = (float)m.kt_c;
        v.damp_cf = (float)m.damp_c;
        v.mu_rollf = (float)m.mu_roll;
        return GDEM_OK;
    }

    TriRecF* trif = nullptr;

    const MeshData* mesh = nullptr;

    void set_mesh(const MeshData& M) override {
        destroy_graphs();
        mesh = &M;
        v.ntri = M.ntri;
        v.tri = M.rec;
        v.seg = M.seg;
        v.segf = M.segf;
        v.seg_tri = M.idx[0];
        v.tri_aabb = M.aabb_d;
        v.seg_top = M.ntri > 0 ? seg_levels(M.ntri) - 1 : 0;
        for (int L = 0; L < kSegMaxLevels; L++) v.seg_off[L] = L <= v.seg_top ? seg_offset_host(M.ntri, L) : 0;
        if (T::mixed) {
            cudaFree(trif);
            trif = nullptr;
            TriLoF* lo = nullptr;
            const size_t hb = sizeof(TriRecF) * (size_t)M.ntri;
            if (M.ntri > 0 && cudaMalloc((void**)&trif, hb + sizeof(TriLoF) * (size_t)M.ntri) == cudaSuccess) {
                lo = reinterpret_cast<TriLoF*>(reinterpret_cast<char*>(trif) + hb);
                launch_trif(M.rec, trif, lo, M.ntri, st);
                cudaStreamSynchronize(st);
            }
            v.trif = trif;
            v.trilo = lo;
            // the FP32 closest-feature distance is within a few ulp of the
            // corner-relative vector (at most the triangle's diagonal plus the
            // radius); 2^-16 of the diagonal bounds that with a wide margin
            v.wall_delta = (float)std::ldexp(M.max_diag, -16);
        }
    }

    // The view the step kernels get: with inner rows, they scan those in
    // place of the list rows.
    View<T> sv() const {
        View<T> s = v;
        if (v.inner_on) {
            s.nei = v.inn;
            s.nnei = v.ninn;
            s.neiw = v.innw;
            s.nneiw = v.ninnw;
        }
        return s;
    }

    int build_graph(int steps, cudaGraphExec_t* out) {
        cudaGraph_t g;
        CKE(cudaGraphCreate(&g, 0));
        cudaGraphNode_t prev = nullptr;
        View<T> vs = sv();
        const bool tree_branch = d.bvh_every_step && mesh && mesh->ntri > 0;
        // the tree rebuild's kernels get CTA slots of their own beside the
        // persistent step kernel, instead of waiting for it to drain
        const StepLaunch L = step_launch(vs, tree_branch ? kTreeReserve : 0);
        for (int k = 0; k < steps; k++) {
            // every handle must belong to a conditional node: the inner-rows
            // handle exists only with inner rows (else the kernel gets hnd twice
            // and leaves the second alone)
            cudaGraphConditionalHandle hnd, hin;
            CKE(cudaGraphConditionalHandleCreate(&hnd, g, 0, cudaGraphCondAssignDefault));
            hin = hnd;
            if (v.inner_on) CKE(cudaGraphConditionalHandleCreate(&hin, g, 0, cudaGraphCondAssignDefault));
            int use_cond = v.inner_on ? 3 : 1;
            void* args[4] = {(void*)&vs, (void*)&hnd, (void*)&hin, (void*)&use_cond};
            cudaKernelNodeParams kp = {};
            kp.func = L.fn;
            kp.gridDim = L.grid;
            kp.blockDim = L.block;
            kp.sharedMemBytes = (unsigned)L.smem;
            kp.kernelParams = args;
            cudaGraphNode_t sn[2];
            int nsn = 1;
            CKE(cudaGraphAddKernelNode(&sn[0], g, prev ? &prev : nullptr, prev ? 1 : 0, &kp));
            if (tree_branch) {
                // the mesh tree rebuild runs beside the step kernel, which
                // reads no part of the tree; the list rebuild that reads it
                // waits for both
                cudaGraph_t bg;
                CKE(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                launch_bvh_rebuild(*mesh, st);
                CKE(cudaStreamEndCapture(st, &bg));
                CKE(cudaGraphAddChildGraphNode(&sn[1], g, prev ? &prev : nullptr, prev ? 1 : 0, bg));
                cudaGraphDestroy(bg);
                nsn = 2;
            }
            cudaGraphNodeParams cp = {};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = hnd;
            cp.conditional.type = cudaGraphCondTypeIf;
            cp.conditional.size = 1;
            cudaGraphNode_t cn;
            CKE(cudaGraphAddNode(&cn, g, sn, nullptr, nsn, &cp));
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            CKE(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal));
            launch_rebuild(v, st, /*force=*/1);
            cudaGraph_t captured;
            CKE(cudaStreamEndCapture(st, &captured));
            prev = cn;
            if (v.inner_on) {
                // new inner rows when some particle moved half the inner skin
                // (after a list rebuild, its own body already made them)
                cudaGraphNodeParams ip = {};
                ip.type = cudaGraphNodeTypeConditional;
                ip.conditional.handle = hin;
                ip.conditional.type = cudaGraphCondTypeIf;
                ip.conditional.size = 1;
                cudaGraphNode_t in;
                CKE(cudaGraphAddNode(&in, g, &prev, nullptr, 1, &ip));
                CKE(cudaStreamBeginCaptureToGraph(st, ip.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeThreadLocal));
                launch_inner(v, st);
                cudaGraph_t cap2;
                CKE(cudaStreamEndCapture(st, &cap2));
                prev = in;
            }
        }
        CKE(cudaGraphInstantiate(out, g, 0));
        cudaGraphDestroy(g);
        return GDEM_OK;
    }

    // x moved into the period [minx, maxx) (periodic x; else unchanged)
    double wrap_x(double x) const {
        if (!v.per_x || !(x >= v.maxx || x < v.minx)) return x;
        x -= v.Lx * floor((x - v.minx) / v.Lx);
        if (x >= v.maxx) x -= v.Lx;
        if (x < v.minx) x += v.Lx;
        return x;
    }

    // Grid, skins and refresh thresholds from the largest radius
    // (initialize_BoundingBox, BoundingBox.cu:370-396).
    int setup_grid(double rmax) {
        const double skin = d.skin > 0 ? d.skin : rmax;
        // FP64 mode keeps the reference's cell (4 r_max) for its bit-exact
        // keys, order and cell lists; mixed mode takes the smallest cell the
        // 27-cell scan allows, the list cutoff 2 r_max + skin, which scans
        // (4 / 3)^3 = 2.4 times fewer candidates at the default skin
        const double cell = d.cell_size > 0 ? d.cell_size : (T::mixed ? 2. * rmax + skin : rmax * 4.);
        const double thresh = d.refresh_thresh > 0 ? d.refresh_thresh : (d.skin > 0 ? skin * 0.5 : rmax * 0.5);
        if (2. * rmax + skin > cell)
            return failv(err, GDEM_ERR_ARG, "cell size smaller than the largest list cutoff 2*r_max+skin");
        v.skin = skin;
        // how far a cell's wall candidates reach: any particle's cutoff
        // r + skin (mixed rows also widen it by the FP32 error bounds), plus a
        // margin far above the rounding of a position's cell coordinate
        v.cw_reach = rmax + skin + (T::mixed ? (double)v.nb_delta + 1e-9 : 0.) + 1e-6 * cell;
        v.thresh_sq = thresh * thresh;
        v.thresh_sqf = (float)v.thresh_sq;
        // inner rows (mixed mode): a tenth of r_max by default, never more than the skin
        v.inner_on = 0;
        v.row_mask = 0xFFFFFFFFu;
        if (T::mixed && d.inner_skin >= 0.) {
            double si = d.inner_skin > 0. ? d.inner_skin : 0.1 * rmax;
            if (si > skin) si = skin;
            v.inner_on = 1;
            v.inner_skin = si;
            if (n < (1 << kHintShift)) v.row_mask = (1u << kHintShift) - 1u;
            v.inner_skinf = (float)si;
            v.inner_thresh_sqf = (float)(0.25 * si * si);
        }
        v.invdx = v.invdy = v.invdz = 1. / cell;
        v.sizex = (int)ceil((v.maxx - v.minx) / cell) + 2;
        if (v.per_x) {
            // whole cells across the period, at least as wide as the cutoff
            v.nxp = (int)floor(v.Lx / cell);
            if (v.nxp < 3) return failv(err, GDEM_ERR_ARG, "periodic x: fewer than 3 cells across the period");
            v.invdx = (double)v.nxp / v.Lx;
            v.sizex = v.nxp + 2;
        }
        v.sizey = (int)ceil((v.maxy - v.miny) / cell) + 2;
        v.sizez = (int)ceil((v.maxz - v.minz) / cell) + 2;
        if (v.sizex > 1024 || v.sizey > 1024 || v.sizez > 1024)
            return failv(err, GDEM_ERR_RANGE, "cell grid exceeds 1024 cells per axis (10-bit Morton keys)");
        v.ncells = v.sizex * v.sizey * v.sizez;
        cudaFree(cell_arena);
        cell_arena = nullptr;
        Arena Cc;
        Cc.add(&v.cell_start, v.ncells);
        Cc.add(&v.cell_end, v.ncells);
        CKE(cudaMalloc((void**)&cell_arena, Cc.total()));
        Cc.bind(cell_arena);
        return GDEM_OK;
    }

    int import_(const gdem_particles* p) override {
        CKE(cudaStreamSynchronize(st));
        destroy_graphs();
        v.per_particle_mat = 0;
        const int H = v.hist_cap, HW = v.histw_cap;
        const bool hist = p->numCont && p->indHis && p->hist_stride > 0;
        const bool histw = p->numContWall && p->indHisWall && p->hist_stride > 0;
        std::vector<int> pid(n), nc(n, 0), ncw(n, 0);
        // history lengths, capacity checks, the slot rows in use, r_max.  The
        // live history keys become device indices (partner particles, mesh
        // triangles), so each is checked here, before anything is uploaded.
        const int ntri = mesh ? mesh->ntri : 0;
        int qmax = 0, qwmax = 0;
        double rmax = 0.;
        // in parallel over contiguous ranges; the first failing range (lowest
        // particles) decides the error
        struct Scan {
            int lo = 0, rc = GDEM_OK, qmax = 0, qwmax = 0;
            double rmax = 0.;
            const char* msg = "";
        };
        std::vector<Scan> scans;
        std::mutex scan_mu;
        host_parallel_for(n, [&](int lo, int hi) {
            Scan sc;
            sc.lo = lo;
            auto bad = [&](int rc, const char* msg) {
                sc.rc = rc;
                sc.msg = msg;
            };
            for (int i = lo; i < hi && sc.rc == GDEM_OK; i++) {
                if (sc.rmax < p->r[i]) sc.rmax = p->r[i];
                if (hist) {
                    nc[i] = p->numCont[i];
                    if (nc[i] < 0) { bad(GDEM_ERR_ARG, "import: negative numCont"); break; }
                    if (nc[i] > H || nc[i] > p->hist_stride) {
                        bad(GDEM_ERR_CAPACITY, "import: history longer than hist_capacity");
                        break;
                    }
                    if (nc[i] > sc.qmax) sc.qmax = nc[i];
                    const int* row = p->indHis + (size_t)i * p->hist_stride;
                    for (int q = 0; q < nc[i]; q++)
                        if (row[q] < 0 || row[q] >= n) {
                            bad(GDEM_ERR_ARG, "import: history partner id outside [0, n)");
                            break;
                        }
                }
                if (histw && sc.rc == GDEM_OK) {
                    ncw[i] = p->numContWall[i];
                    if (ncw[i] < 0) { bad(GDEM_ERR_ARG, "import: negative numContWall"); break; }
                    if (ncw[i] > HW || ncw[i] > p->hist_stride) {
                        bad(GDEM_ERR_CAPACITY, "import: wall history longer than hist_wall_capacity");
                        break;
                    }
                    if (ncw[i] > sc.qwmax) sc.qwmax = ncw[i];
                    const int* row = p->indHisWall + (size_t)i * p->hist_stride;
                    for (int q = 0; q < ncw[i]; q++)
                        if (row[q] < 0 || row[q] >= ntri) {
                            bad(GDEM_ERR_ARG, "import: wall history triangle outside the mesh");
                            break;
                        }
                }
            }
            std::lock_guard<std::mutex> lock(scan_mu);
            scans.push_back(sc);
        });
        std::sort(scans.begin(), scans.end(), [](const Scan& a, const Scan& b) { return a.lo < b.lo; });
        for (const Scan& sc : scans) {
            if (sc.rc != GDEM_OK) return failv(err, sc.rc, sc.msg);
            qmax = std::max(qmax, sc.qmax);
            qwmax = std::max(qwmax, sc.qwmax);
            rmax = std::max(rmax, sc.rmax);
        }
        // staging arrays left uninitialised: the parallel loop below writes
        // every element (first touch spread over the threads)
        HostBuf<double4_32a> pos(n);
        HostBuf<V4> vel(n), rot(n), mat(n);
        HostBuf<float4> posh(T::mixed ? n : 0), posl(T::mixed ? n : 0), vl(T::mixed ? n : 0),
            wl(T::mixed ? n : 0);
        // only the slot rows some particle uses travel; the device clears the rest
        HostBuf<int> hid((size_t)n * qmax), hwid((size_t)n * qwmax);
        HostBuf<R> hx((size_t)n * qmax), hy((size_t)n * qmax), hz((size_t)n * qmax);
        HostBuf<R> hwx((size_t)n * qwmax), hwy((size_t)n * qwmax), hwz((size_t)n * qwmax);
        host_parallel_for(n, [&](int lo, int hi) {
            for (int i = lo; i < hi; i++) {
                const double r = p->r[i];
                pos[i] = make_double4_32a(wrap_x(p->x[3 * i]), p->x[3 * i + 1], p->x[3 * i + 2], r);
                // derived per-particle constants in the operation order of
                // ParticleSystem.cu:294-333 (rsq = r*r, sqrtm, invm, moi = 2/5 m rsq)
                const double rsq = r * r;
                const double sqrtm = sqrt(p->m[i]);
                const double invm = 1. / p->m[i];
                const double moi = 2. / 5. * p->m[i] * rsq;
                const double invmoi = 1. / moi;
                vel[i].x = p->v ? (R)p->v[3 * i] : R(0);
                vel[i].y = p->v ? (R)p->v[3 * i + 1] : R(0);
                vel[i].z = p->v ? (R)p->v[3 * i + 2] : R(0);
                vel[i].w = (R)invm;
                rot[i].x = p->angv ? (R)p->angv[3 * i] : R(0);
                rot[i].y = p->angv ? (R)p->angv[3 * i + 1] : R(0);
                rot[i].z = p->angv ? (R)p->angv[3 * i + 2] : R(0);
                rot[i].w = (R)((p->isActive && p->isActive[i] != 1) ? 0 : 1);
                mat[i].x = (R)p->k[i];
                mat[i].y = (R)p->etaconst[i];
                mat[i].z = (R)sqrtm;
                mat[i].w = (R)invmoi;
                pid[i] = i;
                if (T::mixed) {
                    // float pairs: the FP32 rounding and what it left out
                    const double xs[3] = {pos[i].x, pos[i].y, pos[i].z};
                    float hh[3], ll[3];
                    for (int k = 0; k < 3; k++) {
                        hh[k] = (float)xs[k];
                        ll[k] = (float)(xs[k] - (double)hh[k]);
                    }
                    const float rh = (float)pos[i].w, rl = (float)(pos[i].w - (double)rh);
                    posh[i] = make_float4(hh[0], hh[1], hh[2], rot[i].w == R(1) ? rh : -rh);
                    posl[i] = make_float4(ll[0], ll[1], ll[2], rl);
                    const double vv[3] = {p->v ? p->v[3 * i] : 0., p->v ? p->v[3 * i + 1] : 0.,
                                          p->v ? p->v[3 * i + 2] : 0.};
                    const double ww[3] = {p->angv ? p->angv[3 * i] : 0., p->angv ? p->angv[3 * i + 1] : 0.,
                                          p->angv ? p->angv[3 * i + 2] : 0.};
                    vl[i] = make_float4((float)(vv[0] - (double)vel[i].x), (float)(vv[1] - (double)vel[i].y),
                                        (float)(vv[2] - (double)vel[i].z), 0.f);
                    wl[i] = make_float4((float)(ww[0] - (double)rot[i].x), (float)(ww[1] - (double)rot[i].y),
                                        (float)(ww[2] - (double)rot[i].z), 0.f);
                }
            }
            // slot rows (slot q of particle i at q * n + i): particle by
            // particle, each reading only its live prefix of the source row
            for (int i = lo; i < hi; i++) {
                const size_t row = (size_t)i * p->hist_stride;
                for (int q = 0; q < qmax; q++) {
                    const size_t src = row + q, dst = (size_t)q * n + i;
                    const bool on = q < nc[i];
                    hid[dst] = on ? p->indHis[src] : -1;
                    hx[dst] = on ? (R)p->deltHisx[src] : R(0);
                    hy[dst] = on ? (R)p->deltHisy[src] : R(0);
                    hz[dst] = on ? (R)p->deltHisz[src] : R(0);
                }
                for (int q = 0; q < qwmax; q++) {
                    const size_t src = row + q, dst = (size_t)q * n + i;
                    const bool on = q < ncw[i];
                    hwid[dst] = on ? p->indHisWall[src] : -1;
                    hwx[dst] = on ? (R)p->deltHisxWall[src] : R(0);
                    hwy[dst] = on ? (R)p->deltHisyWall[src] : R(0);
                    hwz[dst] = on ? (R)p->deltHiszWall[src] : R(0);
                }
            }
        });
        if (int rc = setup_grid(rmax)) return rc;
        const SBank<T>& S = v.S[0];
        const PBank<T>& P = v.P[0];
#define UP(dst, src, cnt) \
    if ((cnt) > 0) CKE(cudaMemcpyAsync(dst, src.data(), sizeof(src[0]) * (cnt), cudaMemcpyHostToDevice, st))
        if (!T::mixed) UP(S.pos, pos, n);
        UP(S.vel, vel, n); UP(S.rot, rot, n);
        if (T::mixed) {
            UP(S.posh, posh, n);
            UP(S.posl, posl, n);
            UP(S.vell, vl, n);
            UP(S.rotl, wl, n);
        }
        UP(P.mat, mat, n); UP(P.pid, pid, n);
        UP(P.nc, nc, n); UP(P.hid, hid, (size_t)n * qmax);
        UP(P.hx, hx, (size_t)n * qmax); UP(P.hy, hy, (size_t)n * qmax); UP(P.hz, hz, (size_t)n * qmax);
        UP(P.ncw, ncw, n); UP(P.hwid, hwid, (size_t)n * qwmax);
        UP(P.hwx, hwx, (size_t)n * qwmax); UP(P.hwy, hwy, (size_t)n * qwmax); UP(P.hwz, hwz, (size_t)n * qwmax);
#undef UP
        // the slot rows no particle uses: no key (-1), zero springs
        const size_t r0 = (size_t)n * qmax, r1 = (size_t)n * H, w0 = (size_t)n * qwmax, w1 = (size_t)n * HW;
        if (r1 > r0) {
            CKE(cudaMemsetAsync(P.hid + r0, 0xFF, sizeof(int) * (r1 - r0), st));
            CKE(cudaMemsetAsync(P.hx + r0, 0, sizeof(R) * (r1 - r0), st));
            CKE(cudaMemsetAsync(P.hy + r0, 0, sizeof(R) * (r1 - r0), st));
            CKE(cudaMemsetAsync(P.hz + r0, 0, sizeof(R) * (r1 - r0), st));
        }
        if (w1 > w0) {
            CKE(cudaMemsetAsync(P.hwid + w0, 0xFF, sizeof(int) * (w1 - w0), st));
            CKE(cudaMemsetAsync(P.hwx + w0, 0, sizeof(R) * (w1 - w0), st));
            CKE(cudaMemsetAsync(P.hwy + w0, 0, sizeof(R) * (w1 - w0), st));
            CKE(cudaMemsetAsync(P.hwz + w0, 0, sizeof(R) * (w1 - w0), st));
        }
        if (T::mixed) {
            CKE(cudaMemsetAsync(P.cx, 0, sizeof(R) * (size_t)n * H, st));
            CKE(cudaMemsetAsync(P.cy, 0, sizeof(R) * (size_t)n * H, st));
            CKE(cudaMemsetAsync(P.cz, 0, sizeof(R) * (size_t)n * H, st));
            CKE(cudaMemsetAsync(P.cwx, 0, sizeof(R) * (size_t)n * HW, st));
            CKE(cudaMemsetAsync(P.cwy, 0, sizeof(R) * (size_t)n * HW, st));
            CKE(cudaMemsetAsync(P.cwz, 0, sizeof(R) * (size_t)n * HW, st));
        }
        Ctl c0;
        memset(&c0, 0, sizeof(c0));
        CKE(cudaMemcpyAsync(v.ctl, &c0, sizeof(Ctl), cudaMemcpyHostToDevice, st));
        if (v.store_forces) {
            CKE(cudaMemsetAsync(v.fx, 0, sizeof(double) * n, st));
            CKE(cudaMemsetAsync(v.fy, 0, sizeof(double) * n, st));
            CKE(cudaMemsetAsync(v.fz, 0, sizeof(double) * n, st));
            CKE(cudaMemsetAsync(v.tx, 0, sizeof(double) * n, st));
            CKE(cudaMemsetAsync(v.ty, 0, sizeof(double) * n, st));
            CKE(cudaMemsetAsync(v.tz, 0, sizeof(double) * n, st));
        }
        CKE(cudaStreamSynchronize(st));
        imported = true;
        return rebuild();
    }

    unsigned error_word() override {
        unsigned e = 0;
        cudaMemcpy(&e, &v.ctl->error, sizeof(unsigned), cudaMemcpyDeviceToHost);
        return e;
    }

    int rebuild() override {
        launch_finalize_oob(v, st);
        launch_rebuild(v, st, /*force=*/1);
        CKE(cudaGetLastError());
        CKE(cudaStreamSynchronize(st));
        if (error_word()) return failv(err, GDEM_ERR_DEVICE, "device error word set during rebuild");
        return GDEM_OK;
    }

    int step(int nsteps) override {
        if (!use_graphs) {
            // plain launches: step kernel, then the device-gated rebuild
            for (int q = 0; q < nsteps; q++) {
                launch_step(sv(), st, 0, 0);
                if (d.bvh_every_step && mesh) launch_bvh_rebuild(*mesh, st);
                launch_rebuild(v, st, /*force=*/0);
            }
            CKE(cudaGetLastError());
            return GDEM_OK;
        }
        if (!gK) {
            int rc = build_graph(K, &gK);
            if (rc) return rc;
            rc = build_graph(1, &g1);
            if (rc) return rc;
        }
        const int full = nsteps / K, rest = nsteps % K;
        for (int q = 0; q < full; q++) CKE(cudaGraphLaunch(gK, st));
        for (int q = 0; q < rest; q++) CKE(cudaGraphLaunch(g1, st));
        return GDEM_OK;
    }

    int current(Ctl& c, std::vector<int>& pid) {
        CKE(cudaStreamSynchronize(st));
        CKE(cudaMemcpy(&c, v.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
        pid.resize(n);
        CKE(cudaMemcpy(pid.data(), v.P[c.p].pid, sizeof(int) * n, cudaMemcpyDeviceToHost));
        return GDEM_OK;
    }

    template <typename X>
    int dl(std::vector<X>& out, const X* src, size_t cnt) {
        out.resize(cnt);
        CKE(cudaMemcpy(out.data(), src, sizeof(X) * cnt, cudaMemcpyDeviceToHost));
        return GDEM_OK;
    }

    int export_(gdem_particles* p) override {
        Ctl c;
        std::vector<int> pid;
        int rc = current(c, pid);
        if (rc) return rc;
        const SBank<T>& S = v.S[c.s];
        const PBank<T>& P = v.P[c.p];
        std::vector<double4_32a> pos;
        std::vector<V4> vel, rot, mat;
        if ((rc = dl(vel, S.vel, n)) || (rc = dl(rot, S.rot, n)) || (rc = dl(mat, P.mat, n))) return rc;
        if (T::mixed) {
            std::vector<float4> ph, pl;
            if ((rc = dl(ph, S.posh, n)) || (rc = dl(pl, S.posl, n))) return rc;
            pos.resize(n);
            for (int i = 0; i < n; i++)
                pos[i] = make_double4_32a((double)ph[i].x + (double)pl[i].x, (double)ph[i].y + (double)pl[i].y,
                                          (double)ph[i].z + (double)pl[i].z,
                                          (double)fabsf(ph[i].w) + (double)pl[i].w);
        } else if ((rc = dl(pos, S.pos, n))) {
            return rc;
        }
        std::vector<float4> vl, wl;
        if (T::mixed && ((rc = dl(vl, S.vell, n)) || (rc = dl(wl, S.rotl, n)))) return rc;
        auto lo = [&](const std::vector<float4>& a, int i, int c) -> double {
            if (!T::mixed) return 0.;
            return c == 0 ? a[i].x : (c == 1 ? a[i].y : a[i].z);
        };
        for (int i = 0; i < n; i++) {
            const int q = pid[i];
            if (p->x) { p->x[3 * q] = pos[i].x; p->x[3 * q + 1] = pos[i].y; p->x[3 * q + 2] = pos[i].z; }
            if (p->v) {
                p->v[3 * q] = (double)vel[i].x + lo(vl, i, 0);
                p->v[3 * q + 1] = (double)vel[i].y + lo(vl, i, 1);
                p->v[3 * q + 2] = (double)vel[i].z + lo(vl, i, 2);
            }
            if (p->angv) {
                p->angv[3 * q] = (double)rot[i].x + lo(wl, i, 0);
                p->angv[3 * q + 1] = (double)rot[i].y + lo(wl, i, 1);
                p->angv[3 * q + 2] = (double)rot[i].z + lo(wl, i, 2);
            }
            if (p->isActive) p->isActive[q] = rot[i].w == R(1) ? 1 : 0;
            if (p->r) p->r[q] = pos[i].w;
            if (p->m) p->m[q] = 1. / (double)vel[i].w;
            if (p->k) p->k[q] = mat[i].x;
            if (p->etaconst) p->etaconst[q] = mat[i].y;
        }
        if (p->f || p->mom) {
            if (!v.store_forces) return failv(err, GDEM_ERR_STATE, "forces not stored (store_forces=0)");
            std::vector<double> a, b, cc;
            auto vec3 = [&](double* out, const double* X, const double* Y, const double* Z) -> int {
                int r2 = dl(a, X, n) | dl(b, Y, n) | dl(cc, Z, n);
                if (r2) return r2;
                for (int i = 0; i < n; i++) {
                    out[3 * pid[i]] = a[i];
                    out[3 * pid[i] + 1] = b[i];
                    out[3 * pid[i] + 2] = cc[i];
                }
                return 0;
            };
            if (p->f && (rc = vec3(p->f, v.fx, v.fy, v.fz))) return rc;
            if (p->mom && (rc = vec3(p->mom, v.tx, v.ty, v.tz))) return rc;
        }
        const int stv = p->hist_stride;
        auto hist = [&](int* cnt, int* ind, double* X, double* Y, double* Z, const int* dn, const int* did,
                        const R* dx, const R* dy, const R* dz, int cap) -> int {
            std::vector<int> nc, id;
            std::vector<R> hx, hy, hz;
            int r2;
            if ((r2 = dl(nc, dn, n)) || (r2 = dl(id, did, (size_t)n * cap)) || (r2 = dl(hx, dx, (size_t)n * cap)) ||
                (r2 = dl(hy, dy, (size_t)n * cap)) || (r2 = dl(hz, dz, (size_t)n * cap)))
                return r2;
            for (int i = 0; i < n; i++) {
                const int q = pid[i];
                cnt[q] = nc[i];
                for (int s2 = 0; s2 < nc[i] && s2 < stv; s2++) {
                    const size_t src = (size_t)s2 * n + i, dst = (size_t)q * stv + s2;
                    // mixed-mode particle keys are storage indices: report pIds
                    if (ind) ind[dst] = (T::mixed && did == P.hid) ? pid[id[src]] : id[src];
                    if (X) X[dst] = hx[src];
                    if (Y) Y[dst] = hy[src];
                    if (Z) Z[dst] = hz[src];
                }
            }
            return 0;
        };
        if (p->numCont && stv > 0 &&
            (rc = hist(p->numCont, p->indHis, p->deltHisx, p->deltHisy, p->deltHisz, P.nc, P.hid, P.hx, P.hy,
                       P.hz, v.hist_cap)))
            return rc;
        if (p->numContWall && stv > 0 &&
            (rc = hist(p->numContWall, p->indHisWall, p->deltHisxWall, p->deltHisyWall, p->deltHiszWall, P.ncw,
                       P.hwid, P.hwx, P.hwy, P.hwz, v.histw_cap)))
            return rc;
        return GDEM_OK;
    }

    int export_positions(double* x) override {
        launch_gather_positions(v, gather, st);
        CKE(cudaMemcpyAsync(x, gather, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost, st));
        CKE(cudaStreamSynchronize(st));
        return GDEM_OK;
    }

    // Positions in pId order into host memory without waiting: the gather
    // runs on the engine's stream, the copy on the copy stream after it, so
    // the steps launched next overlap the transfer.  Two device buffers take
    // turns; a buffer is gathered into again only after its last copy ended.
    double* pgather[2] = {nullptr, nullptr};
    cudaEvent_t pready[2] = {nullptr, nullptr}, pcopied[2] = {nullptr, nullptr};
    int pslot = 0;

    int export_positions_async(double* x) override {
        if (!pgather[0]) {
            if (!copy_st) CKE(cudaStreamCreateWithFlags(&copy_st, cudaStreamNonBlocking));
            for (int k = 0; k < 2; k++) {
                CKE(cudaMalloc((void**)&pgather[k], sizeof(double) * 3 * (size_t)n));
                CKE(cudaEventCreateWithFlags(&pready[k], cudaEventDisableTiming));
                CKE(cudaEventCreateWithFlags(&pcopied[k], cudaEventDisableTiming));
                CKE(cudaEventRecord(pcopied[k], copy_st));
            }
        }
        const int k = pslot;
        pslot ^= 1;
        CKE(cudaStreamWaitEvent(st, pcopied[k], 0));
        launch_gather_positions(v, pgather[k], st);
        CKE(cudaGetLastError());
        CKE(cudaEventRecord(pready[k], st));
        CKE(cudaStreamWaitEvent(copy_st, pready[k], 0));
        CKE(cudaMemcpyAsync(x, pgather[k], sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost, copy_st));
        CKE(cudaEventRecord(pcopied[k], copy_st));
        return GDEM_OK;
    }

    int sync_copies() override {
        if (copy_st) CKE(cudaStreamSynchronize(copy_st));
        return GDEM_OK;
    }

    int lists(int stride, int* numNei, int* neiList, int* numNeiWall, int* neiListWall) override {
        Ctl c;
        std::vector<int> pid;
        int rc = current(c, pid);
        if (rc) return rc;
        std::vector<int> cnt, rows;
        if (numNei || neiList) {
            if ((rc = dl(cnt, (const int*)v.nnei, n)) || (rc = dl(rows, (const int*)v.nei, (size_t)n * v.nei_cap)))
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
            if ((rc = dl(cnt, (const int*)v.nneiw, n)) ||
                (rc = dl(rows, (const int*)v.neiw, (size_t)n * v.wall_cap)))
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

    int keys(uint32_t* out) override {
        launch_keys_probe(v, v.keys[1], st);
        CKE(cudaGetLastError());
        Ctl c;
        std::vector<int> pid;
        int rc = current(c, pid);
        if (rc) return rc;
        std::vector<uint32_t> k;
        if ((rc = dl(k, (const uint32_t*)v.keys[1], n))) return rc;
        for (int i = 0; i < n; i++) out[pid[i]] = k[i];
        return GDEM_OK;
    }

    int cells(uint32_t* keys_sorted, int* order, int* pNum, int* pStart, int* pList, int* n_cells) override {
        if (n_cells) *n_cells = v.ncells;
        if (!keys_sorted && !order && !pNum && !pStart && !pList) return GDEM_OK;
        Ctl c;
        std::vector<int> pid;
        int rc = current(c, pid);
        if (rc) return rc;
        std::vector<uint32_t> k;
        std::vector<int> vals, cs, ce;
        if ((rc = dl(k, (const uint32_t*)v.keys[0], n)) || (rc = dl(vals, (const int*)v.vals[0], n)) ||
            (rc = dl(cs, (const int*)v.cell_start, v.ncells)) || (rc = dl(ce, (const int*)v.cell_end, v.ncells)))
            return rc;
        if (keys_sorted) memcpy(keys_sorted, k.data(), sizeof(uint32_t) * n);
        std::vector<int> at(n);
        for (int q = 0; q < n; q++) at[q] = v.reorder ? q : vals[q];
        if (order)
            for (int q = 0; q < n; q++) order[q] = pid[at[q]];
        int run = 0;
        for (int cc = 0; cc < v.ncells; cc++) {
            const int cnt = ce[cc] - cs[cc];
            if (pNum) pNum[cc] = cnt;
            if (pStart) pStart[cc] = run;
            if (pList)
                for (int t = 0; t < cnt; t++) pList[run + t] = at[cs[cc] + t];
            run += cnt;
        }
        return GDEM_OK;
    }

    int stats(gdem_stats* s) override {
        launch_stats(v, stats_partials, stats_nblk, st);
        CKE(cudaGetLastError());
        CKE(cudaStreamSynchronize(st));
        std::vector<double> part((size_t)16 * stats_nblk);
        CKE(cudaMemcpy(part.data(), stats_partials, sizeof(double) * part.size(), cudaMemcpyDeviceToHost));
        Ctl c;
        CKE(cudaMemcpy(&c, v.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
        double acc[7] = {0, 0, 0, 0, 0, 0, 0};
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, mo = 0., ninn_sum = 0., ninnw_sum = 0.;
        for (int b = 0; b < stats_nblk; b++) {
            const double* q = &part[(size_t)16 * b];
            for (int k = 0; k < 7; k++) acc[k] += q[k];
            for (int k = 0; k < 3; k++) {
                lo[k] = std::min(lo[k], q[7 + k]);
                hi[k] = std::max(hi[k], q[10 + k]);
            }
            mo = std::max(mo, q[13]);
            ninn_sum += q[14];
            ninnw_sum += q[15];
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
        s->n_inner = (long long)ninn_sum;
        s->inner_builds = (long long)c.inner_builds;
        s->n_inner_wall = (long long)ninnw_sum;
        return GDEM_OK;
    }

    // Hertz-Mindlin friction and damping per particle (pId order), written
    // into the material records of the current property bank.
    int set_materials(const double* mu, const double* restitution) override {
        if (d.model != GDEM_HERTZ_MINDLIN)
            return failv(err, GDEM_ERR_STATE, "per-particle materials need the Hertz-Mindlin model");
        Ctl c;
        std::vector<int> pid;
        int rc = current(c, pid);
        if (rc) return rc;
        std::vector<V4> mat;
        if ((rc = dl(mat, v.P[c.p].mat, n))) return rc;
        for (int i = 0; i < n; i++) {
            const int q = pid[i];
            const double e = restitution[q];
            if (!(e > 0. && e <= 1.) || !(mu[q] >= 0.))
                return failv(err, GDEM_ERR_ARG, "restitution must be in (0, 1] and friction >= 0");
            const double le = log(e);
            const double beta = le / sqrt(le * le + M_PI * M_PI);
            mat[i].x = (R)mu[q];
            mat[i].y = (R)(-2. * sqrt(5. / 6.) * beta);
        }
        CKE(cudaMemcpy(v.P[c.p].mat, mat.data(), sizeof(V4) * n, cudaMemcpyHostToDevice));
        destroy_graphs();
        v.per_particle_mat = 1;
        return GDEM_OK;
    }

    // ---------------------------------------------------------------- frames
    // write_frame_bin payloads built on the device (gdem_output.cu), copied to
    // pinned host buffers on a copy stream after the frame kernels, and
    // written to files by a host thread: the steps launched after a frame run
    // while it travels and lands.  Three buffers; a fourth frame waits for one.
    struct FrameSlot {
        char* dev = nullptr;
        char* host = nullptr;
        cudaEvent_t ready = nullptr, copied = nullptr;
        bool busy = false;
    };
    struct FrameJob {
        int slot;
        std::string path;
    };
    static constexpr int kFrameSlots = 3;
    FrameSlot fslot[kFrameSlots];
    void* fscratch = nullptr;
    cudaStream_t copy_st = nullptr;
    std::thread fwriter;
    std::mutex fmu;
    std::condition_variable fcv;
    std::deque<FrameJob> fjobs;
    bool fstop = false;
    int fpending = 0;
    std::string ferr;

    int frames_init() {
        if (fscratch) return GDEM_OK;
        CKE(cudaMalloc(&fscratch, frame_scratch_bytes(n)));
        if (!copy_st) CKE(cudaStreamCreateWithFlags(&copy_st, cudaStreamNonBlocking));
        const size_t fb = frame_bytes(n);
        for (auto& s : fslot) {
            CKE(cudaMalloc((void**)&s.dev, fb));
            CKE(cudaHostAlloc((void**)&s.host, fb, cudaHostAllocDefault));
            CKE(cudaEventCreateWithFlags(&s.ready, cudaEventDisableTiming));
            CKE(cudaEventCreateWithFlags(&s.copied, cudaEventDisableTiming));
        }
        fwriter = std::thread([this] { frame_writer(); });
        return GDEM_OK;
    }

    void frame_writer() {
        for (;;) {
            FrameJob job;
            {
                std::unique_lock<std::mutex> lk(fmu);
                fcv.wait(lk, [this] { return fstop || !fjobs.empty(); });
                if (fjobs.empty()) return;
                job = fjobs.front();
                fjobs.pop_front();
            }
            FrameSlot& s = fslot[job.slot];
            std::string e;
            if (cudaEventSynchronize(s.copied) != cudaSuccess) {
                e = "frame copy failed";
            } else {
                int count = 0;
                memcpy(&count, s.host, 4);
                FILE* fp = fopen(job.path.c_str(), "wb");
                if (!fp) {
                    e = "cannot open " + job.path;
                } else {
                    const size_t bytes = 4 + 16 * (size_t)count;
                    if (fwrite(s.host, 1, bytes, fp) != bytes) e = "short write to " + job.path;
                    if (fclose(fp) != 0 && e.empty()) e = "cannot close " + job.path;
                }
            }
            {
                std::lock_guard<std::mutex> lk(fmu);
                if (!e.empty() && ferr.empty()) ferr = e;
                s.busy = false;
                fpending--;
            }
            fcv.notify_all();
        }
    }

    void frames_shutdown() {
        if (!fscratch) return;
        {
            std::lock_guard<std::mutex> lk(fmu);
            fstop = true;
        }
        fcv.notify_all();
        if (fwriter.joinable()) fwriter.join();
        for (auto& s : fslot) {
            cudaFree(s.dev);
            cudaFreeHost(s.host);
            if (s.ready) cudaEventDestroy(s.ready);
            if (s.copied) cudaEventDestroy(s.copied);
        }
        cudaFree(fscratch);
        fscratch = nullptr;
    }

    int frame_async(const char* dir, int step, double lf) override {
        if (!dir) return failv(err, GDEM_ERR_ARG, "frame: null directory");
        int rc = frames_init();
        if (rc) return rc;
        int k = -1;
        {
            std::unique_lock<std::mutex> lk(fmu);
            fcv.wait(lk, [this] {
                for (auto& s : fslot)
                    if (!s.busy) return true;
                return false;
            });
            for (int q = 0; q < kFrameSlots && k < 0; q++)
                if (!fslot[q].busy) k = q;
            fslot[k].busy = true;
            fpending++;
        }
        FrameSlot& s = fslot[k];
        launch_frame(v, fscratch, s.dev, lf, st);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(s.ready, st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(copy_st, s.ready, 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(s.host, s.dev, frame_bytes(n), cudaMemcpyDeviceToHost, copy_st);
        if (e == cudaSuccess) e = cudaEventRecord(s.copied, copy_st);
        if (e != cudaSuccess) {
            {
                std::lock_guard<std::mutex> lk(fmu);
                s.busy = false;
                fpending--;
            }
            fcv.notify_all();
            return failv(err, GDEM_ERR_CUDA, std::string("frame: ") + cudaGetErrorString(e));
        }
        char name[64];
        snprintf(name, sizeof(name), "/result_%012d.bin", step);
        {
            std::lock_guard<std::mutex> lk(fmu);
            fjobs.push_back(FrameJob{k, std::string(dir) + name});
        }
        fcv.notify_all();
        return GDEM_OK;
    }

    int frames_flush() override {
        std::string e;
        {
            std::unique_lock<std::mutex> lk(fmu);
            fcv.wait(lk, [this] { return fpending == 0; });
            e.swap(ferr);
        }
        if (!e.empty()) return failv(err, GDEM_ERR_ARG, e);
        return GDEM_OK;
    }

    // ---------------------------------------------------------------- device init
    int init_particles(const gdem_inlet* in) override {
        double* buf = nullptr;
        CKE(cudaMalloc((void**)&buf, sizeof(double) * 10 * (size_t)n));
        double *dx = buf, *dv = buf + 3 * (size_t)n, *dr = buf + 6 * (size_t)n, *dm = buf + 7 * (size_t)n,
               *dk = buf + 8 * (size_t)n, *de = buf + 9 * (size_t)n;
        std::string msg;
        int rc = init_particles_device(*in, n, dx, dv, dr, dm, dk, de, st, msg);
        std::vector<double> h((size_t)10 * n);
        if (rc == GDEM_OK && cudaMemcpy(h.data(), buf, sizeof(double) * h.size(), cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = GDEM_ERR_CUDA;
            msg = "init: copy of the particles failed";
        }
        cudaFree(buf);
        if (rc) return failv(err, rc, msg);
        gdem_particles pp;
        memset(&pp, 0, sizeof(pp));
        pp.n = n;
        pp.x = h.data();
        pp.v = h.data() + 3 * (size_t)n;
        pp.r = h.data() + 6 * (size_t)n;
        pp.m = h.data() + 7 * (size_t)n;
        pp.k = h.data() + 8 * (size_t)n;
        pp.etaconst = h.data() + 9 * (size_t)n;
        return import_(&pp);
    }

    // ---------------------------------------------------------------- snapshot
    // The exact state in pId order: the precision's own representation of
    // positions, velocities, spins (float pairs in mixed mode) and material
    // records, and the compact contact histories with partners as pIds (all
    // spring terms).  Loading it into an engine of the same size, precision
    // and model (with its mesh set) continues the run bit for bit: storage
    // order, lists and rebuild times differ, and none of them enters the
    // results.
    int save_snapshot(const char* path) override {
        if (!path) return failv(err, GDEM_ERR_ARG, "snapshot: null path");
        Ctl c;
        std::vector<int> pid;
        int rc = current(c, pid);
        if (rc) return rc;
        const SBank<T>& S = v.S[c.s];
        const PBank<T>& P = v.P[c.p];
        const int H = v.hist_cap, HW = v.histw_cap;
        std::vector<int> at(n);
        for (int i = 0; i < n; i++) at[pid[i]] = i;
        std::vector<V4> vel, rot, mat;
        std::vector<double4_32a> pos;
        std::vector<float4> ph, pl, vl, wl;
        std::vector<int> nc, ncw, hid, hwid;
        std::vector<R> hh[6], hw[6];
        if ((rc = dl(vel, S.vel, n)) || (rc = dl(rot, S.rot, n)) || (rc = dl(mat, P.mat, n)) ||
            (rc = dl(nc, P.nc, n)) || (rc = dl(ncw, P.ncw, n)) || (rc = dl(hid, P.hid, (size_t)n * H)) ||
            (rc = dl(hwid, P.hwid, (size_t)n * HW)))
            return rc;
        R* const hsrc[6] = {P.hx, P.hy, P.hz, P.cx, P.cy, P.cz};
        R* const wsrc[6] = {P.hwx, P.hwy, P.hwz, P.cwx, P.cwy, P.cwz};
        const int nterms = T::mixed ? 6 : 3;
        for (int a = 0; a < nterms; a++)
            if ((rc = dl(hh[a], hsrc[a], (size_t)n * H)) || (rc = dl(hw[a], wsrc[a], (size_t)n * HW))) return rc;
        if (T::mixed) {
            if ((rc = dl(ph, S.posh, n)) || (rc = dl(pl, S.posl, n)) || (rc = dl(vl, S.vell, n)) ||
                (rc = dl(wl, S.rotl, n)))
                return rc;
        } else if ((rc = dl(pos, S.pos, n))) {
            return rc;
        }
        FILE* fp = fopen(path, "wb");
        if (!fp) return failv(err, GDEM_ERR_ARG, std::string("snapshot: cannot open ") + path);
        bool ok = true;
        auto put = [&](const void* p, size_t bytes) {
            if (ok && fwrite(p, 1, bytes, fp) != bytes) ok = false;
        };
        SnapHeader hd;
        memset(&hd, 0, sizeof(hd));
        memcpy(hd.magic, "GDEMSNAP", 8);
        hd.version = 1;
        hd.n = n;
        hd.precision = T::mixed ? GDEM_MIXED : GDEM_FP64;
        hd.model = d.model;
        hd.hist_cap = H;
        hd.histw_cap = HW;
        hd.per_particle_mat = v.per_particle_mat;
        hd.rsize = (int)sizeof(R);
        hd.steps = c.steps;
        hd.error = c.error;
        put(&hd, sizeof(hd));
        auto put_perm = [&](const auto& a) {
            using E = typename std::decay<decltype(a)>::type::value_type;
            std::vector<E> o(n);
            for (int q = 0; q < n; q++) o[q] = a[at[q]];
            put(o.data(), sizeof(E) * o.size());
        };
        if (T::mixed) {
            put_perm(ph); put_perm(pl); put_perm(vel); put_perm(vl); put_perm(rot); put_perm(wl);
        } else {
            put_perm(pos); put_perm(vel); put_perm(rot);
        }
        put_perm(mat);
        // histories: counts, then each particle's live entries (partner pId or
        // triangle, then the spring terms)
        auto put_hist = [&](const std::vector<int>& cnt, const std::vector<int>& id, std::vector<R>* terms,
                            bool partner_is_particle) {
            put_perm(cnt);
            std::vector<int> ids;
            std::vector<R> vals;
            for (int q = 0; q < n; q++) {
                const int i = at[q];
                for (int k = 0; k < cnt[i]; k++) {
                    const size_t s = (size_t)k * n + i;
                    int key = id[s];
                    if (partner_is_particle && T::mixed) key = pid[key];  // storage index -> pId
                    ids.push_back(key);
                    for (int a = 0; a < nterms; a++) vals.push_back(terms[a][s]);
                }
            }
            put(ids.data(), sizeof(int) * ids.size());
            put(vals.data(), sizeof(R) * vals.size());
        };
        put_hist(nc, hid, hh, true);
        put_hist(ncw, hwid, hw, false);
        if (fclose(fp) != 0) ok = false;
        if (!ok) return failv(err, GDEM_ERR_ARG, std::string("snapshot: cannot write ") + path);
        return GDEM_OK;
    }

    int load_snapshot(const char* path) override {
        if (!path) return failv(err, GDEM_ERR_ARG, "snapshot: null path");
        {
            std::string msg;
            if (int rc = check_snapshot_file(path, mesh ? mesh->ntri : 0, nullptr, msg)) return failv(err, rc, msg);
        }
        FILE* fp = fopen(path, "rb");
        if (!fp) return failv(err, GDEM_ERR_ARG, std::string("snapshot: cannot open ") + path);
        bool ok = true;
        auto get = [&](void* p, size_t bytes) {
            if (ok && fread(p, 1, bytes, fp) != bytes) ok = false;
        };
        SnapHeader hd;
        get(&hd, sizeof(hd));
        const int H = v.hist_cap, HW = v.histw_cap;
        if (!ok || memcmp(hd.magic, "GDEMSNAP", 8) != 0 || hd.version != 1) {
            fclose(fp);
            return failv(err, GDEM_ERR_ARG, "snapshot: not a snapshot file");
        }
        if (hd.n != n || hd.precision != (T::mixed ? GDEM_MIXED : GDEM_FP64) || hd.model != d.model ||
            hd.rsize != (int)sizeof(R)) {
            fclose(fp);
            return failv(err, GDEM_ERR_ARG, "snapshot: size, precision or model differs from this engine");
        }
        std::vector<V4> vel(n), rot(n), mat(n);
        std::vector<double4_32a> pos;
        std::vector<float4> ph, pl, vl, wl;
        if (T::mixed) {
            ph.resize(n); pl.resize(n); vl.resize(n); wl.resize(n);
            get(ph.data(), 16 * (size_t)n); get(pl.data(), 16 * (size_t)n);
            get(vel.data(), sizeof(V4) * (size_t)n); get(vl.data(), 16 * (size_t)n);
            get(rot.data(), sizeof(V4) * (size_t)n); get(wl.data(), 16 * (size_t)n);
        } else {
            pos.resize(n);
            get(pos.data(), sizeof(double4_32a) * (size_t)n);
            get(vel.data(), sizeof(V4) * (size_t)n);
            get(rot.data(), sizeof(V4) * (size_t)n);
        }
        get(mat.data(), sizeof(V4) * (size_t)n);
        const int nterms = T::mixed ? 6 : 3;
        std::vector<int> nc(n), ncw(n), ids, idsw;
        std::vector<R> vals, valsw;
        // every history key becomes a device index (a partner particle or a
        // mesh triangle): a key outside [0, id_end) refuses the file before
        // anything is uploaded
        bool ids_ok = true;
        auto get_hist = [&](std::vector<int>& cnt, std::vector<int>& id, std::vector<R>& val, int cap, int id_end) {
            get(cnt.data(), sizeof(int) * (size_t)n);
            size_t tot = 0;
            for (int q = 0; q < n && ok; q++) {
                if (cnt[q] < 0 || cnt[q] > cap) ok = false;
                tot += (size_t)cnt[q];
            }
            if (!ok) return;
            id.resize(tot);
            val.resize(tot * nterms);
            get(id.data(), sizeof(int) * tot);
            get(val.data(), sizeof(R) * val.size());
            for (size_t e = 0; e < tot && ok; e++)
                if (id[e] < 0 || id[e] >= id_end) ids_ok = false;
        };
        get_hist(nc, ids, vals, H, n);
        get_hist(ncw, idsw, valsw, HW, mesh ? mesh->ntri : 0);
        fclose(fp);
        if (!ok) return failv(err, GDEM_ERR_ARG, "snapshot: truncated, or a history longer than this engine's capacity");
        if (!ids_ok)
            return failv(err, GDEM_ERR_ARG, "snapshot: a history key outside the particles or the mesh triangles");
        // set the engine up as an import would (grid, lists), from the
        // reference-layout view of the snapshot ...
        std::vector<double> x(3 * (size_t)n), vv(3 * (size_t)n), ww(3 * (size_t)n), r(n), m(n), k(n), eta(n);
        std::vector<int> act(n);
        for (int q = 0; q < n; q++) {
            double xs[4];
            if (T::mixed) {
                xs[0] = (double)ph[q].x + (double)pl[q].x;
                xs[1] = (double)ph[q].y + (double)pl[q].y;
                xs[2] = (double)ph[q].z + (double)pl[q].z;
                xs[3] = (double)fabsf(ph[q].w) + (double)pl[q].w;
            } else {
                xs[0] = pos[q].x; xs[1] = pos[q].y; xs[2] = pos[q].z; xs[3] = pos[q].w;
            }
            for (int a = 0; a < 3; a++) x[3 * q + a] = xs[a];
            r[q] = xs[3];
            vv[3 * q] = (double)vel[q].x; vv[3 * q + 1] = (double)vel[q].y; vv[3 * q + 2] = (double)vel[q].z;
            ww[3 * q] = (double)rot[q].x; ww[3 * q + 1] = (double)rot[q].y; ww[3 * q + 2] = (double)rot[q].z;
            m[q] = 1. / (double)vel[q].w;
            k[q] = (double)mat[q].x;
            eta[q] = (double)mat[q].y;
            act[q] = rot[q].w == R(1) ? 1 : 0;
        }
        gdem_particles pp;
        memset(&pp, 0, sizeof(pp));
        pp.n = n;
        pp.x = x.data(); pp.v = vv.data(); pp.angv = ww.data(); pp.r = r.data(); pp.m = m.data();
        pp.k = k.data(); pp.etaconst = eta.data(); pp.isActive = act.data();
        int rc = import_(&pp);
        if (rc) return rc;
        // ... then put the exact state into the current banks, in the storage
        // order the import's rebuild chose
        Ctl c;
        std::vector<int> pid;
        if ((rc = current(c, pid))) return rc;
        std::vector<int> at(n);
        for (int i = 0; i < n; i++) at[pid[i]] = i;
        const SBank<T>& S = v.S[c.s];
        const PBank<T>& P = v.P[c.p];
        auto up_perm = [&](auto* dst, const auto& a) -> int {
            using E = typename std::decay<decltype(a)>::type::value_type;
            std::vector<E> o(n);
            for (int q = 0; q < n; q++) o[at[q]] = a[q];
            CKE(cudaMemcpy(dst, o.data(), sizeof(E) * (size_t)n, cudaMemcpyHostToDevice));
            return GDEM_OK;
        };
        if (T::mixed) {
            if ((rc = up_perm(S.posh, ph)) || (rc = up_perm(S.posl, pl)) || (rc = up_perm(S.vell, vl)) ||
                (rc = up_perm(S.rotl, wl)))
                return rc;
        } else if ((rc = up_perm(S.pos, pos))) {
            return rc;
        }
        if ((rc = up_perm(S.vel, vel)) || (rc = up_perm(S.rot, rot)) || (rc = up_perm(P.mat, mat))) return rc;
        auto up_hist = [&](const std::vector<int>& cnt, const std::vector<int>& id, const std::vector<R>& val,
                           int cap, int* dcnt, int* did, R* const* dterm, bool partner_is_particle) -> int {
            std::vector<int> c2(n, 0), id2((size_t)n * cap, -1);
            std::vector<R> t2[6];
            for (int a = 0; a < nterms; a++) t2[a].assign((size_t)n * cap, R(0));
            size_t e = 0;
            for (int q = 0; q < n; q++) {
                const int i = at[q];
                c2[i] = cnt[q];
                for (int kk = 0; kk < cnt[q]; kk++, e++) {
                    const size_t s = (size_t)kk * n + i;
                    int key = id[e];
                    if (partner_is_particle && T::mixed) key = at[key];  // pId -> storage index
                    id2[s] = key;
                    for (int a = 0; a < nterms; a++) t2[a][s] = val[e * nterms + a];
                }
            }
            CKE(cudaMemcpy(dcnt, c2.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice));
            CKE(cudaMemcpy(did, id2.data(), sizeof(int) * id2.size(), cudaMemcpyHostToDevice));
            for (int a = 0; a < nterms; a++)
                CKE(cudaMemcpy(dterm[a], t2[a].data(), sizeof(R) * t2[a].size(), cudaMemcpyHostToDevice));
            return GDEM_OK;
        };
        R* const hdst[6] = {P.hx, P.hy, P.hz, P.cx, P.cy, P.cz};
        R* const wdst[6] = {P.hwx, P.hwy, P.hwz, P.cwx, P.cwy, P.cwz};
        if ((rc = up_hist(nc, ids, vals, H, P.nc, P.hid, hdst, true)) ||
            (rc = up_hist(ncw, idsw, valsw, HW, P.ncw, P.hwid, wdst, false)))
            return rc;
        v.per_particle_mat = hd.per_particle_mat;
        destroy_graphs();
        c.steps = hd.steps;
        c.error = hd.error;
        CKE(cudaMemcpy(v.ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice));
        return rebuild();
    }

    int profile(int iters, float* avg_ms) override {
        // groups of kProfileBurst launches back to back between two events;
        // the device-gated rebuild runs after each group
        constexpr int kProfileBurst = 4;
        const int groups = (iters + kProfileBurst - 1) / kProfileBurst;
        std::vector<cudaEvent_t> ev(2 * groups);
        for (auto& e : ev) CKE(cudaEventCreate(&e));
        for (int q = 0; q < groups; q++) {
            CKE(cudaEventRecord(ev[2 * q], st));
            for (int b = 0; b < kProfileBurst; b++) launch_step(sv(), st, 0, 0);
            CKE(cudaEventRecord(ev[2 * q + 1], st));
            launch_rebuild(v, st, /*force=*/0);
        }
        CKE(cudaStreamSynchronize(st));
        CKE(cudaGetLastError());
        double tot = 0.;
        for (int q = 0; q < groups; q++) {
            float ms = 0.f;
            CKE(cudaEventElapsedTime(&ms, ev[2 * q], ev[2 * q + 1]));
            tot += ms;
        }
        iters = groups * kProfileBurst;
        for (auto& e : ev) cudaEventDestroy(e);
        *avg_ms = (float)(tot / iters);
        return GDEM_OK;
    }
};

}  // namespace

struct gdem_handle {
    gdem_desc d;
    std::unique_ptr<EngineBase> eng;
    MeshData mesh;
    std::string err;
};

namespace {

int fail(gdem_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    return code;
}

int pass(gdem_handle* h, int rc) {
    if (rc != GDEM_OK && h) h->err = h->eng->err;
    return rc;
}

#define CK(call)                                                                            \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(h, GDEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

extern "C" {

const char* gdem_last_error(gdem_handle* h) { return h ? h->err.c_str() : "null handle"; }

int gdem_create(const gdem_desc* desc, gdem_handle** out) {
    if (!desc || !out) return GDEM_ERR_ARG;
    if (desc->n_particles <= 0) return GDEM_ERR_ARG;
    if (desc->precision != GDEM_FP64 && desc->precision != GDEM_MIXED) return GDEM_ERR_ARG;
    if (desc->model != GDEM_LINEAR && desc->model != GDEM_HERTZ_MINDLIN) return GDEM_ERR_ARG;
    gdem_desc d = *desc;
    if (d.nei_capacity <= 0) d.nei_capacity = 64;
    if (d.wall_capacity <= 0) d.wall_capacity = 32;
    if (d.hist_capacity <= 0) d.hist_capacity = 32;
    if (d.hist_wall_capacity <= 0) d.hist_wall_capacity = 16;
    if (d.steps_per_graph <= 0) d.steps_per_graph = 8;
    if (d.nei_capacity > 128 || d.wall_capacity > 64 || d.hist_capacity > 64 || d.hist_wall_capacity > 64)
        return GDEM_ERR_ARG;
    if (d.model == GDEM_HERTZ_MINDLIN &&
        !(d.youngs_modulus > 0 && d.poisson_ratio > -1 && d.poisson_ratio < 0.5 && d.restitution > 0 &&
          d.restitution <= 1))
        return GDEM_ERR_ARG;
    gdem_handle* h = new gdem_handle();
    h->d = d;
    int rc;
    if (d.precision == GDEM_MIXED) {
        auto* e = new Impl<Mixed>();
        h->eng.reset(e);
        rc = e->create(d);
    } else {
        auto* e = new Impl<FP64>();
        h->eng.reset(e);
        rc = e->create(d);
    }
    if (rc != GDEM_OK) {
        delete h;
        return rc;
    }
    *out = h;
    return GDEM_OK;
}

int gdem_destroy(gdem_handle* h) {
    if (!h) return GDEM_ERR_ARG;
    h->eng.reset();
    cudaFree(h->mesh.arena);
    delete h;
    return GDEM_OK;
}

// ---------------------------------------------------------------- mesh
static int upload_mesh(gdem_handle* h, const std::vector<double>& vx, const std::vector<double>& vy,
                       const std::vector<double>& vz, const std::vector<int>& tv, const std::vector<int>& te,
                       const double* raw3_h, const double* dplane_h, int T);

int gdem_set_mesh(gdem_handle* h, const double* tris, int n_tri, const int* file_tri_counts, int nfiles) {
    if (!h || n_tri < 0 || (n_tri > 0 && !tris)) return fail(h, GDEM_ERR_ARG, "bad mesh arguments");
    cudaStream_t st = h->eng->st;
    cudaStreamSynchronize(st);
    MeshData& M = h->mesh;
    if (n_tri == 0) {
        cudaFree(M.arena);
        M = MeshData();
        h->eng->set_mesh(M);
        return h->eng->imported ? pass(h, h->eng->rebuild()) : GDEM_OK;
    }
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
            unsigned long long hh = 1469598103934665603ULL;
            hh ^= (unsigned long long)k.x; hh *= 1099511628211ULL;
            hh ^= (unsigned long long)k.y; hh *= 1099511628211ULL;
            hh ^= (unsigned long long)k.z; hh *= 1099511628211ULL;
            return (size_t)hh;
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
                const double x = tris[9 * t + 3 * c], y = tris[9 * t + 3 * c + 1], z = tris[9 * t + 3 * c + 2];
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
                const unsigned long long key = ((unsigned long long)(unsigned)pairs[q][0] << 32) | (unsigned)pairs[q][1];
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
    return upload_mesh(h, vx, vy, vz, tv, te, raw3.data(), nullptr, T);
}

// Device half of the mesh set-up, shared by gdem_set_mesh (welded here) and
// gdem_set_mesh_indexed (welded by the caller's loader): triangle and mesh
// AABBs, per-triangle records, centroid keys, their sort and the mesh tree.  The
// plane offset comes from the raw third corner (raw3) or is given (dplane).
static int upload_mesh(gdem_handle* h, const std::vector<double>& vx, const std::vector<double>& vy,
                       const std::vector<double>& vz, const std::vector<int>& tv, const std::vector<int>& te,
                       const double* raw3_h, const double* dplane_h, int T) {
    cudaStream_t st = h->eng->st;
    MeshData& M = h->mesh;
    // ---- a corrupt mesh is refused before anything reaches the device:
    // non-finite coordinates or plane offsets, and triangles of zero area
    // (their unit normal, n = e01 x e02 / |e01 x e02|, does not exist)
    for (size_t q = 0; q < vx.size(); q++)
        if (!std::isfinite(vx[q]) || !std::isfinite(vy[q]) || !std::isfinite(vz[q]))
            return fail(h, GDEM_ERR_ARG, "mesh: a vertex coordinate is NaN or infinite");
    for (int t = 0; t < T; t++) {
        if (raw3_h && !(std::isfinite(raw3_h[3 * t]) && std::isfinite(raw3_h[3 * t + 1]) &&
                        std::isfinite(raw3_h[3 * t + 2])))
            return fail(h, GDEM_ERR_ARG, "mesh: a triangle corner is NaN or infinite");
        if (dplane_h && !std::isfinite(dplane_h[t])) return fail(h, GDEM_ERR_ARG, "mesh: a plane offset is NaN or infinite");
        const int a = tv[3 * t], b = tv[3 * t + 1], c = tv[3 * t + 2];
        const double e1[3] = {vx[b] - vx[a], vy[b] - vy[a], vz[b] - vz[a]};
        const double e2[3] = {vx[c] - vx[a], vy[c] - vy[a], vz[c] - vz[a]};
        const double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                              e1[0] * e2[1] - e1[1] * e2[0]};
        if (cr[0] == 0. && cr[1] == 0. && cr[2] == 0.)
            return fail(h, GDEM_ERR_ARG, "mesh: a triangle has zero area (repeated or collinear corners)");
        if (h->d.periodic_x) {
            const double L = h->d.box_max[0] - h->d.box_min[0];
            const double w = std::max(vx[a], std::max(vx[b], vx[c])) - std::min(vx[a], std::min(vx[b], vx[c]));
            if (!(w < 0.25 * L)) return fail(h, GDEM_ERR_ARG, "periodic x: a triangle is wider than a quarter period");
        }
    }
    if (T > (1 << kSegShift)) return fail(h, GDEM_ERR_ARG, "mesh: more than 2^26 triangles");
    // the mesh is sound: the previous one (if any) goes
    cudaFree(M.arena);
    M = MeshData();
    // ---- triangle AABBs and the mesh AABB, in the loader's comparison order
    M.aabb_h.assign(6 * (size_t)T, 0.);
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
            M.aabb_h[6 * t + k] = mn;
            M.aabb_h[6 * t + 3 + k] = mx;
        }
        for (int k = 0; k < 3; k++)
            if (M.aabb_h[6 * t + k] < g[k]) g[k] = M.aabb_h[6 * t + k];
        for (int k = 0; k < 3; k++)
            if (M.aabb_h[6 * t + 3 + k] > g[3 + k]) g[3 + k] = M.aabb_h[6 * t + 3 + k];
        double d2 = 0.;
        for (int k = 0; k < 3; k++) {
            const double e = M.aabb_h[6 * t + 3 + k] - M.aabb_h[6 * t + k];
            d2 += e * e;
        }
        if (d2 > M.max_diag * M.max_diag) M.max_diag = std::sqrt(d2);
    }
    const int SCALE = (1 << 10) - 1;
    double inv[3];
    for (int k = 0; k < 3; k++) inv[k] = SCALE / (g[3 + k] - g[k]);
    // ---- device side: precompute records, centroid keys, sort, mesh tree
    const int NV = (int)vx.size();
    Arena A;
    double *dvx, *dvy, *dvz, *draw3;
    int *dtv, *dte;
    const int nb = rs_blocks_for(T);
    A.add(&M.rec, T);
    A.add(&M.aabb_d, 6 * (size_t)T);
    A.add(&dvx, NV); A.add(&dvy, NV); A.add(&dvz, NV);
    A.add(&draw3, raw3_h ? 3 * (size_t)T : (size_t)T);
    A.add(&dtv, 3 * (size_t)T); A.add(&dte, 3 * (size_t)T);
    A.add(&M.seg, bvh_scratch_bytes(T) / sizeof(SegBox));
    A.add(&M.segf, bvh_scratch_bytes(T) / sizeof(SegBox));
    A.add(&M.done, 1);
    A.add(&M.morton[0], T); A.add(&M.morton[1], T);
    A.add(&M.idx[0], T); A.add(&M.idx[1], T);
    A.add(&M.hist, (size_t)256 * nb);
    A.add(&M.tot, 256);
    CK(cudaMalloc((void**)&M.arena, A.total()));
    A.bind(M.arena);
    CK(cudaMemsetAsync(M.done, 0, sizeof(unsigned), st));
    M.ntri = T;
    CK(cudaMemcpyAsync(dvx, vx.data(), sizeof(double) * NV, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dvy, vy.data(), sizeof(double) * NV, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dvz, vz.data(), sizeof(double) * NV, cudaMemcpyHostToDevice, st));
    if (raw3_h)
        CK(cudaMemcpyAsync(draw3, raw3_h, sizeof(double) * 3 * T, cudaMemcpyHostToDevice, st));
    else
        CK(cudaMemcpyAsync(draw3, dplane_h, sizeof(double) * T, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dtv, tv.data(), sizeof(int) * 3 * T, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dte, te.data(), sizeof(int) * 3 * T, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(M.aabb_d, M.aabb_h.data(), sizeof(double) * 6 * T, cudaMemcpyHostToDevice, st));
    launch_tri_precompute(M.rec, M.morton[0], M.idx[0], dvx, dvy, dvz, dtv, dte, raw3_h ? draw3 : nullptr,
                          raw3_h ? nullptr : draw3, T, g, inv, st);
    // stable sort of the centroid keys (radixSortUint32 at TriangleMesh.cu:722)
    for (int k = 0; k < 3; k++) {
        M.gmin[k] = g[k];
        M.ginv[k] = inv[k];
    }
    radix_sort_pairs(M.morton[0], M.idx[0], M.morton[1], M.idx[1], M.hist, M.tot, T, nb, 0, 4, st);
    launch_bvh_build(M.aabb_d, M.idx[0], M.seg, M.segf, M.done, T, st);
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    h->eng->set_mesh(M);
    if (h->eng->imported) return pass(h, h->eng->rebuild());
    return GDEM_OK;
}

int gdem_set_mesh_indexed(gdem_handle* h, const gdem_mesh_arrays* m) {
    if (!h || !m || m->nTri < 0 || m->nVert < 0) return fail(h, GDEM_ERR_ARG, "bad mesh arguments");
    const int T = m->nTri, NV = m->nVert;
    if (T > 0 && (!m->mx || !m->my || !m->mz || !m->tri_i0 || !m->tri_i1 || !m->tri_i2 || !m->tri_e0 ||
                  !m->tri_e1 || !m->tri_e2 || !m->d))
        return fail(h, GDEM_ERR_ARG, "mesh arrays missing");
    cudaStreamSynchronize(h->eng->st);
    MeshData& M = h->mesh;
    if (T == 0) {
        cudaFree(M.arena);
        M = MeshData();
        h->eng->set_mesh(M);
        return h->eng->imported ? pass(h, h->eng->rebuild()) : GDEM_OK;
    }
    std::vector<double> vx(m->mx, m->mx + NV), vy(m->my, m->my + NV), vz(m->mz, m->mz + NV);
    std::vector<int> tv(3 * (size_t)T), te(3 * (size_t)T);
    for (int t = 0; t < T; t++) {
        const int a = m->tri_i0[t], b = m->tri_i1[t], c = m->tri_i2[t];
        // the loader stores each triangle's vertex ids ascending (sort3, TriangleMesh.cu:89-103)
        if (a < 0 || c >= NV || a > b || b > c) return fail(h, GDEM_ERR_ARG, "need 0 <= tri_i0 <= tri_i1 <= tri_i2 < nVert");
        if (m->tri_e0[t] < 0 || m->tri_e1[t] < 0 || m->tri_e2[t] < 0)
            return fail(h, GDEM_ERR_ARG, "mesh: negative edge id");
        tv[3 * t] = a; tv[3 * t + 1] = b; tv[3 * t + 2] = c;
        te[3 * t] = m->tri_e0[t]; te[3 * t + 1] = m->tri_e1[t]; te[3 * t + 2] = m->tri_e2[t];
    }
    return upload_mesh(h, vx, vy, vz, tv, te, nullptr, m->d, T);
}

int gdem_export_mesh(gdem_handle* h, double* rec, int* irec, double* aabb, uint32_t* morton, int* sorted_index) {
    if (!h) return GDEM_ERR_ARG;
    const MeshData& M = h->mesh;
    const int T = M.ntri;
    if (T == 0) return GDEM_OK;
    CK(cudaStreamSynchronize(h->eng->st));
    std::vector<TriRec> R(T);
    CK(cudaMemcpy(R.data(), M.rec, sizeof(TriRec) * T, cudaMemcpyDeviceToHost));
    for (int t = 0; t < T; t++) {
        if (rec) memcpy(rec + 29 * (size_t)t, &R[t], 29 * sizeof(double));
        if (irec) memcpy(irec + 6 * (size_t)t, &R[t].i0, 6 * sizeof(int));
    }
    if (aabb) memcpy(aabb, M.aabb_h.data(), sizeof(double) * 6 * T);
    if (morton) CK(cudaMemcpy(morton, M.morton[0], sizeof(uint32_t) * T, cudaMemcpyDeviceToHost));
    if (sorted_index) CK(cudaMemcpy(sorted_index, M.idx[0], sizeof(int) * T, cudaMemcpyDeviceToHost));
    return GDEM_OK;
}

// ---------------------------------------------------------------- particles
int gdem_import_particles(gdem_handle* h, const gdem_particles* p) {
    if (!h || !p || p->n != h->d.n_particles || !p->x || !p->r || !p->m || !p->k || !p->etaconst)
        return fail(h, GDEM_ERR_ARG, "import: missing arrays or wrong n");
    return pass(h, h->eng->import_(p));
}

int gdem_rebuild(gdem_handle* h) {
    if (!h || !h->eng->imported) return fail(h, GDEM_ERR_STATE, "rebuild before import");
    return pass(h, h->eng->rebuild());
}

int gdem_step(gdem_handle* h, int nsteps) {
    if (!h || !h->eng->imported) return fail(h, GDEM_ERR_STATE, "step before import");
    if (nsteps < 0) return fail(h, GDEM_ERR_ARG, "negative step count");
    return pass(h, h->eng->step(nsteps));
}

int gdem_export_positions_async(gdem_handle* h, double* x) {
    if (!h || !x) return fail(h, GDEM_ERR_ARG, "export_positions_async: null");
    if (!h->eng->imported) return fail(h, GDEM_ERR_STATE, "export before import");
    return pass(h, h->eng->export_positions_async(x));
}

int gdem_synchronize(gdem_handle* h) {
    if (!h) return GDEM_ERR_ARG;
    CK(cudaStreamSynchronize(h->eng->st));
    if (int rc = pass(h, h->eng->sync_copies())) return rc;
    CK(cudaGetLastError());
    if (h->eng->error_word()) return fail(h, GDEM_ERR_DEVICE, "device error word set");
    return GDEM_OK;
}

int gdem_export_particles(gdem_handle* h, gdem_particles* p) {
    if (!h || !p || p->n != h->d.n_particles) return fail(h, GDEM_ERR_ARG, "export: wrong n");
    if (!h->eng->imported) return fail(h, GDEM_ERR_STATE, "export before import");
    return pass(h, h->eng->export_(p));
}

int gdem_frame_write_async(gdem_handle* h, const char* dir, int step, double length_factor) {
    if (!h || !dir) return fail(h, GDEM_ERR_ARG, "frame_write_async: null");
    if (!h->eng->imported) return fail(h, GDEM_ERR_STATE, "frame before import");
    return pass(h, h->eng->frame_async(dir, step, length_factor));
}

int gdem_init_particles(gdem_handle* h, const gdem_inlet* in) {
    if (!h || !in) return fail(h, GDEM_ERR_ARG, "init_particles: null");
    if (in->placement != GDEM_PLACE_RANDOM && in->placement != GDEM_PLACE_LATTICE)
        return fail(h, GDEM_ERR_ARG, "init_particles: unknown placement");
    if (in->radius_dist < GDEM_RADIUS_MONO || in->radius_dist > GDEM_RADIUS_BIDISPERSE)
        return fail(h, GDEM_ERR_ARG, "init_particles: unknown radius distribution");
    if (!(in->r_a > 0) || (in->radius_dist != GDEM_RADIUS_MONO && !(in->r_b > 0)) ||
        (in->radius_dist == GDEM_RADIUS_LOGNORMAL && !(in->r_c > 0 && in->r_d >= in->r_c)) ||
        !(in->density > 0) || !(in->restitution > 0 && in->restitution <= 1) || !(in->youngs_modulus > 0))
        return fail(h, GDEM_ERR_ARG, "init_particles: bad radius, density or material");
    for (int a = 0; a < 3; a++)
        if (!(in->box_max[a] > in->box_min[a])) return fail(h, GDEM_ERR_ARG, "init_particles: empty region");
    const int rc = pass(h, h->eng->init_particles(in));
    if (rc == GDEM_OK) h->eng->imported = true;
    return rc;
}

int gdem_frames_flush(gdem_handle* h) {
    if (!h) return GDEM_ERR_ARG;
    return pass(h, h->eng->frames_flush());
}

int gdem_save_snapshot(gdem_handle* h, const char* path) {
    if (!h || !path) return fail(h, GDEM_ERR_ARG, "save_snapshot: null");
    if (!h->eng->imported) return fail(h, GDEM_ERR_STATE, "snapshot before import");
    return pass(h, h->eng->save_snapshot(path));
}

int gdem_load_snapshot(gdem_handle* h, const char* path) {
    if (!h || !path) return fail(h, GDEM_ERR_ARG, "load_snapshot: null");
    const int rc = pass(h, h->eng->load_snapshot(path));
    if (rc == GDEM_OK) h->eng->imported = true;
    return rc;
}

int gdem_check_snapshot(const char* path, int n_tri) {
    if (!path || n_tri < 0) return GDEM_ERR_ARG;
    std::string msg;
    return check_snapshot_file(path, n_tri, nullptr, msg);
}

int gdem_export_positions(gdem_handle* h, double* x) {
    if (!h || !x) return fail(h, GDEM_ERR_ARG, "export_positions: null");
    if (!h->eng->imported) return fail(h, GDEM_ERR_STATE, "export before import");
    return pass(h, h->eng->export_positions(x));
}

int gdem_export_lists(gdem_handle* h, int stride, int* numNei, int* neiList, int* numNeiWall, int* neiListWall) {
    if (!h || stride <= 0) return fail(h, GDEM_ERR_ARG, "export_lists: bad stride");
    if (!h->eng->imported) return fail(h, GDEM_ERR_STATE, "export before import");
    return pass(h, h->eng->lists(stride, numNei, neiList, numNeiWall, neiListWall));
}

int gdem_morton_keys(gdem_handle* h, uint32_t* keys) {
    if (!h || !keys) return fail(h, GDEM_ERR_ARG, "morton_keys: null");
    if (!h->eng->imported) return fail(h, GDEM_ERR_STATE, "keys before import");
    return pass(h, h->eng->keys(keys));
}

int gdem_export_cells(gdem_handle* h, uint32_t* keys_sorted, int* order, int* pNum, int* pStart, int* pList,
                      int* n_cells) {
    if (!h) return GDEM_ERR_ARG;
    if (!h->eng->imported) return fail(h, GDEM_ERR_STATE, "cells before import");
    return pass(h, h->eng->cells(keys_sorted, order, pNum, pStart, pList, n_cells));
}

int gdem_stats_get(gdem_handle* h, gdem_stats* s) {
    if (!h || !s) return GDEM_ERR_ARG;
    if (!h->eng->imported) return fail(h, GDEM_ERR_STATE, "stats before import");
    return pass(h, h->eng->stats(s));
}

int gdem_set_particle_materials(gdem_handle* h, const double* mu, const double* restitution) {
    if (!h || !mu || !restitution) return GDEM_ERR_ARG;
    if (!h->eng->imported) return fail(h, GDEM_ERR_STATE, "materials before import");
    return pass(h, h->eng->set_materials(mu, restitution));
}

int gdem_get_stream(gdem_handle* h, void** stream) {
    if (!h || !stream) return GDEM_ERR_ARG;
    *stream = (void*)h->eng->st;
    return GDEM_OK;
}

int gdem_profile_step(gdem_handle* h, int iters, float* avg_ms) {
    if (!h || iters <= 0 || !avg_ms) return GDEM_ERR_ARG;
    if (!h->eng->imported) return fail(h, GDEM_ERR_STATE, "profile before import");
    return pass(h, h->eng->profile(iters, avg_ms));
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

int gdem_dist_triangle(gdem_handle* h, const double* pos, const double* r, const int* tri, int m, double* out4,
                       int* hitAt) {
    if (!h || m < 0) return GDEM_ERR_ARG;
    if (m == 0) return GDEM_OK;
    if (h->mesh.ntri == 0) return fail(h, GDEM_ERR_STATE, "no mesh");
    for (int q = 0; q < m; q++)
        if (tri[q] < 0 || tri[q] >= h->mesh.ntri) return fail(h, GDEM_ERR_ARG, "triangle index out of range");
    cudaStream_t st = h->eng->st;
    Arena A;
    double *dp, *dr, *dout;
    int *dt, *dh;
    A.add(&dp, 3 * (size_t)m); A.add(&dr, m); A.add(&dt, m); A.add(&dout, 4 * (size_t)m); A.add(&dh, m);
    char* base;
    CK(cudaMalloc((void**)&base, A.total()));
    A.bind(base);
    cudaMemcpyAsync(dp, pos, sizeof(double) * 3 * m, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dr, r, sizeof(double) * m, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dt, tri, sizeof(int) * m, cudaMemcpyHostToDevice, st);
    launch_dist_triangle(h->mesh.rec, dp, dr, dt, m, dout, dh, st);
    cudaMemcpyAsync(out4, dout, sizeof(double) * 4 * m, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(hitAt, dh, sizeof(int) * m, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(base);
    if (e != cudaSuccess) return fail(h, GDEM_ERR_CUDA, cudaGetErrorString(e));
    return GDEM_OK;
}

}  // extern "C"
