// Reference-side binding of libgdem.so for gpudem's GPU main loop.
//
// Add this file to gpudem's source tree and build it with the reference's
// own flags plus the engine's header, then link the engine:
//
//   nvcc -O3 -DUSE_GPU=1 -arch=sm_103a -I<this repo>/include -c gdem_device_dem.cu
//   nvcc ... main.o ... gdem_device_dem.o -L<this repo>/gpudem_gb300/_build -lgdem
//
// and change two calls in main.cu:
//   main.cu:270  device_dem_verlet_verlet(&d_ps, &box, &mesh, &bvh, gridSize, blockSize);
//            ->  gdem_device_dem_verlet_verlet(&d_ps, &box, &mesh, &bvh, gridSize, blockSize);
//   main.cu:279  copyFromDevice(&d_ps, &ps);
//            ->  gdem_copy_from_device(&d_ps, &ps);
//
// The first step call creates the engine from what the reference has already
// set up: the particle arrays copyToDevice uploaded (ParticleSystem.cu:82),
// the box limits, cell size, skin and refresh threshold of
// initialize_BoundingBox (BoundingBox.cu:377-389) and the welded mesh of
// load_ascii_stl_double (TriangleMesh.cu:363).  From then on the engine owns
// the state; the reference's device arrays are no longer advanced, so every
// read of the state goes through gdem_copy_from_device.
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "BVH.h"
#include "BoundingBox.h"
#include "ParticleSystem.h"
#include "TriangleMesh.h"
#include "gdem.h"

static gdem_handle* g_engine = nullptr;

static void gdem_check(int rc, const char* what) {
    if (rc == GDEM_OK) return;
    fprintf(stderr, "%s failed (%d): %s\n", what, rc, g_engine ? gdem_last_error(g_engine) : "");
    exit(1);
}

template <class T>
static std::vector<T> to_host(const T* d, size_t n) {
    std::vector<T> h(n);
    if (cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost) != cudaSuccess) {
        fprintf(stderr, "gdem shim: device read failed\n");
        exit(1);
    }
    return h;
}

static void gdem_bind(ParticleSys<DeviceMemory>* p, BoundingBox* box, TriangleMesh* mesh) {
    const int N = p->N;
    const size_t H = (size_t)N * MAX_NEI;
    gdem_desc d = {};
    d.n_particles = N;
    d.precision = GDEM_FP64;  // GDEM_MIXED for the FP32-contact mode
    d.model = GDEM_LINEAR;
    d.nei_capacity = MAX_NEI;
    d.wall_capacity = 64;
    d.hist_capacity = 64;
    d.hist_wall_capacity = 64;
    d.reorder = 1;
    d.dt = p->dt;
    d.mu = p->mu;
    const std::vector<double> g = to_host(p->g, DIM);
    for (int c = 0; c < 3; c++) d.g[c] = g[c];
    d.box_min[0] = box->minx; d.box_min[1] = box->miny; d.box_min[2] = box->minz;
    d.box_max[0] = box->maxx; d.box_max[1] = box->maxy; d.box_max[2] = box->maxz;
    d.cell_size = box->dx;
    d.skin = box->skinR;
    d.refresh_thresh = box->refreshThresh;
    gdem_check(gdem_create(&d, &g_engine), "gdem_create");

    gdem_mesh_arrays m = {};
    m.nVert = mesh->nVert;
    m.nTri = mesh->nTri;
    m.mx = mesh->mx; m.my = mesh->my; m.mz = mesh->mz;
    m.tri_i0 = mesh->tri_i0; m.tri_i1 = mesh->tri_i1; m.tri_i2 = mesh->tri_i2;
    m.tri_e0 = mesh->tri_e0; m.tri_e1 = mesh->tri_e1; m.tri_e2 = mesh->tri_e2;
    m.d = mesh->d;
    gdem_check(gdem_set_mesh_indexed(g_engine, &m), "gdem_set_mesh_indexed");

    std::vector<double> x = to_host(p->x, 3 * (size_t)N), v = to_host(p->v, 3 * (size_t)N),
                        w = to_host(p->angv, 3 * (size_t)N), r = to_host(p->r, N), mass = to_host(p->m, N),
                        k = to_host(p->k, N), eta = to_host(p->etaconst, N);
    std::vector<int> act = to_host(p->isActive, N), nc = to_host(p->numCont, N),
                     ih = to_host(p->indHis, H), ncw = to_host(p->numContWall, N),
                     ihw = to_host(p->indHisWall, H);
    std::vector<double> hx = to_host(p->deltHisx, H), hy = to_host(p->deltHisy, H), hz = to_host(p->deltHisz, H),
                        hwx = to_host(p->deltHisxWall, H), hwy = to_host(p->deltHisyWall, H),
                        hwz = to_host(p->deltHiszWall, H);
    gdem_particles q = {};
    q.n = N;
    q.x = x.data(); q.v = v.data(); q.angv = w.data();
    q.r = r.data(); q.m = mass.data(); q.k = k.data(); q.etaconst = eta.data();
    q.isActive = act.data();
    q.hist_stride = MAX_NEI;
    q.numCont = nc.data(); q.indHis = ih.data();
    q.deltHisx = hx.data(); q.deltHisy = hy.data(); q.deltHisz = hz.data();
    q.numContWall = ncw.data(); q.indHisWall = ihw.data();
    q.deltHisxWall = hwx.data(); q.deltHisyWall = hwy.data(); q.deltHiszWall = hwz.data();
    gdem_check(gdem_import_particles(g_engine, &q), "gdem_import_particles");
}

// Same parameters as device_dem_verlet_verlet (device_dem.h:112); the BVH
// and launch shape are unused: the engine keeps its own LBVH and launch
// configuration.
void gdem_device_dem_verlet_verlet(ParticleSys<DeviceMemory>* p, BoundingBox* box, TriangleMesh* mesh, BVH* bvh,
                                   int gridSize, int blockSize) {
    (void)bvh;
    (void)gridSize;
    (void)blockSize;
    if (!g_engine) gdem_bind(p, box, mesh);
    gdem_check(gdem_step(g_engine, 1), "gdem_step");
}

// Same parameters as copyFromDevice (ParticleSystem.cu:97): fills the
// SAVE_ON fields write_frame_bin and write_single_text read, in pId order.
void gdem_copy_from_device(ParticleSys<DeviceMemory>* d_ps, ParticleSys<HostMemory>* ps) {
    (void)d_ps;
    gdem_check(gdem_synchronize(g_engine), "gdem_synchronize");
    gdem_particles q = {};
    q.n = ps->N;
    q.x = ps->x; q.v = ps->v; q.angv = ps->angv;
    q.isActive = ps->isActive;
    q.hist_stride = MAX_NEI;
    q.numCont = ps->numCont; q.indHis = ps->indHis;
    q.deltHisx = ps->deltHisx; q.deltHisy = ps->deltHisy; q.deltHisz = ps->deltHisz;
    q.numContWall = ps->numContWall; q.indHisWall = ps->indHisWall;
    q.deltHisxWall = ps->deltHisxWall; q.deltHisyWall = ps->deltHisyWall; q.deltHiszWall = ps->deltHiszWall;
    gdem_check(gdem_export_particles(g_engine, &q), "gdem_export_particles");
}
