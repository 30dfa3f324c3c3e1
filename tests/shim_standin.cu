// Test driver for the reference-side binding's body (gdem_shim_core.h) on a
// GPU where the reference's sources are not present.  The structs below have
// the members the binding reads, with the reference's names, types and
// layouts (ParticleSystem.h / memberList/ParticleSystemMember_common.def,
// BoundingBox.h, TriangleMesh.h); the particle arrays live on the device in
// the reference's row layout (xyz-interleaved vectors, MAX_NEI-strided
// history rows), filled as copyToDevice (ParticleSystem.cu:82) leaves them
// after initializeParticles (ParticleSystem.cu:294-335).  Built and loaded by
// tests/test_shim_gpu.py only.
#include <cuda_runtime.h>
#include <string.h>

#include <vector>

#include "gdem.h"
#include "gdem_shim_core.h"

namespace {

constexpr int kMaxNei = 100;  // MAX_NEI, hardCodedParameters.h:3

struct StandinParticles {  // ParticleSysShared: scalars, then member arrays
    double dt, mu;
    int N;
    double *x, *v, *angv, *r, *m, *k, *etaconst, *g;
    int* isActive;
    double *deltHisx, *deltHisy, *deltHisz, *deltHisxWall, *deltHisyWall, *deltHiszWall;
    int *indHis, *indHisWall, *numCont, *numContWall;
};
struct StandinBox {
    double minx, miny, minz, maxx, maxy, maxz, dx, skinR, refreshThresh;
};
struct StandinMesh {
    int nVert, nTri;
    double *mx, *my, *mz;
    int *tri_i0, *tri_i1, *tri_i2, *tri_e0, *tri_e1, *tri_e2;
    double* d;
};

StandinParticles g_dev, g_host;
StandinBox g_box;
StandinMesh g_mesh;
std::vector<double> g_mesh_d[4];
std::vector<int> g_mesh_i[6];

template <class T>
int up(T** dst, const T* src, size_t n) {
    if (cudaMalloc((void**)dst, sizeof(T) * (n ? n : 1)) != cudaSuccess) return GDEM_ERR_CUDA;
    if (n && cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice) != cudaSuccess) return GDEM_ERR_CUDA;
    return GDEM_OK;
}

}  // namespace

extern "C" {

// Particles (pId order, no contact history yet), the BoundingBox values
// initialize_BoundingBox computed (minx..maxz, dx, skinR, refreshThresh) and
// the loader's welded mesh arrays.
int standin_setup(int N, const double* x, const double* v, const double* w, const double* r, const double* m,
                  const double* k, const double* eta, double dt, double mu, const double* g, const double* box9,
                  int nVert, int nTri, const double* mx, const double* my, const double* mz, const int* ti0,
                  const int* ti1, const int* ti2, const int* te0, const int* te1, const int* te2, const double* d) {
    memset(&g_dev, 0, sizeof(g_dev));
    g_dev.dt = dt;
    g_dev.mu = mu;
    g_dev.N = N;
    const size_t H = (size_t)N * kMaxNei;
    std::vector<int> act(N, 1), zero(N, 0), minus1(H, -1);
    std::vector<double> dzero(H, 0.);
    int rc;
    if ((rc = up(&g_dev.x, x, 3 * (size_t)N)) || (rc = up(&g_dev.v, v, 3 * (size_t)N)) ||
        (rc = up(&g_dev.angv, w, 3 * (size_t)N)) || (rc = up(&g_dev.r, r, N)) || (rc = up(&g_dev.m, m, N)) ||
        (rc = up(&g_dev.k, k, N)) || (rc = up(&g_dev.etaconst, eta, N)) || (rc = up(&g_dev.g, g, 3)) ||
        (rc = up(&g_dev.isActive, act.data(), N)) || (rc = up(&g_dev.numCont, zero.data(), N)) ||
        (rc = up(&g_dev.numContWall, zero.data(), N)) || (rc = up(&g_dev.indHis, minus1.data(), H)) ||
        (rc = up(&g_dev.indHisWall, minus1.data(), H)) || (rc = up(&g_dev.deltHisx, dzero.data(), H)) ||
        (rc = up(&g_dev.deltHisy, dzero.data(), H)) || (rc = up(&g_dev.deltHisz, dzero.data(), H)) ||
        (rc = up(&g_dev.deltHisxWall, dzero.data(), H)) || (rc = up(&g_dev.deltHisyWall, dzero.data(), H)) ||
        (rc = up(&g_dev.deltHiszWall, dzero.data(), H)))
        return rc;
    g_box = StandinBox{box9[0], box9[1], box9[2], box9[3], box9[4], box9[5], box9[6], box9[7], box9[8]};
    g_mesh_d[0].assign(mx, mx + nVert);
    g_mesh_d[1].assign(my, my + nVert);
    g_mesh_d[2].assign(mz, mz + nVert);
    g_mesh_d[3].assign(d, d + nTri);
    const int* ti[6] = {ti0, ti1, ti2, te0, te1, te2};
    for (int a = 0; a < 6; a++) g_mesh_i[a].assign(ti[a], ti[a] + nTri);
    g_mesh = StandinMesh{nVert, nTri, g_mesh_d[0].data(), g_mesh_d[1].data(), g_mesh_d[2].data(),
                         g_mesh_i[0].data(), g_mesh_i[1].data(), g_mesh_i[2].data(), g_mesh_i[3].data(),
                         g_mesh_i[4].data(), g_mesh_i[5].data(), g_mesh_d[3].data()};
    return GDEM_OK;
}

// nsteps calls of the binding's device_dem_verlet_verlet replacement.
int standin_step(int nsteps) {
    for (int s = 0; s < nsteps; s++) {
        const int rc = gdem_shim::step(&g_dev, &g_box, &g_mesh, kMaxNei);
        if (rc) {
            gdem_shim::report(rc, "standin step");
            return rc;
        }
    }
    return GDEM_OK;
}

// The binding's copyFromDevice replacement into caller-owned host rows
// (history arrays [N * MAX_NEI]).
int standin_copy_back(double* x, double* v, double* angv, int* isActive, int* numCont, int* indHis, double* hx,
                      double* hy, double* hz, int* numContWall, int* indHisWall, double* hwx, double* hwy,
                      double* hwz) {
    memset(&g_host, 0, sizeof(g_host));
    g_host.N = g_dev.N;
    g_host.x = x; g_host.v = v; g_host.angv = angv; g_host.isActive = isActive;
    g_host.numCont = numCont; g_host.indHis = indHis;
    g_host.deltHisx = hx; g_host.deltHisy = hy; g_host.deltHisz = hz;
    g_host.numContWall = numContWall; g_host.indHisWall = indHisWall;
    g_host.deltHisxWall = hwx; g_host.deltHisyWall = hwy; g_host.deltHiszWall = hwz;
    return gdem_shim::copy_from_device(&g_host, kMaxNei);
}

int standin_release() {
    double** dp[] = {&g_dev.x, &g_dev.v, &g_dev.angv, &g_dev.r, &g_dev.m, &g_dev.k, &g_dev.etaconst, &g_dev.g,
                     &g_dev.deltHisx, &g_dev.deltHisy, &g_dev.deltHisz, &g_dev.deltHisxWall, &g_dev.deltHisyWall,
                     &g_dev.deltHiszWall};
    int** ip[] = {&g_dev.isActive, &g_dev.indHis, &g_dev.indHisWall, &g_dev.numCont, &g_dev.numContWall};
    for (auto p : dp) { cudaFree(*p); *p = nullptr; }
    for (auto p : ip) { cudaFree(*p); *p = nullptr; }
    return gdem_shim::release();
}

}  // extern "C"
