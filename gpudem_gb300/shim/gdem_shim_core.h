// Body of the reference-side binding (gdem_device_dem.cu), written against
// the member names of gpudem's structs and nothing else, so it compiles with
// the reference's own ParticleSys<DeviceMemory>, BoundingBox and TriangleMesh
// (ParticleSystem.h, BoundingBox.h, TriangleMesh.h) and with any struct that
// has the same members.
//
// What it reads, as the reference lays it out:
//  * particles: the scalars dt, mu, N of ParticleSysShared and the device
//    arrays of memberList/ParticleSystemMember_common.def that the step needs
//    (x, v, angv [3N]; r, m, k, etaconst, isActive, numCont, numContWall [N];
//    g [3]; indHis, deltHis{x,y,z}, indHisWall, deltHis{x,y,z}Wall [N*max_nei]);
//  * box: minx..maxz, dx (cell size), skinR, refreshThresh
//    (initialize_BoundingBox, BoundingBox.cu:377-389);
//  * mesh: nVert, nTri, mx/my/mz, tri_i0..2, tri_e0..2, d, the welded arrays
//    of load_ascii_stl_double (TriangleMesh.cu:363-752), on the host.
// Every function returns a gdem status code; the reference-side wrappers turn
// a failure into a message (with the device error word's bits) and exit, as
// the reference's own host code aborts on errors.
#ifndef GDEM_SHIM_CORE_H
#define GDEM_SHIM_CORE_H

#include <cuda_runtime.h>
#include <stdio.h>

#include <vector>

#include "gdem.h"

namespace gdem_shim {

// One engine per process, created by the first step call.
inline gdem_handle*& engine() {
    static gdem_handle* h = nullptr;
    return h;
}

// Engine settings the binding chooses (the reference has no counterpart).
struct Options {
    int precision = GDEM_FP64;  // GDEM_MIXED for the FP32-contact mode
    int model = GDEM_LINEAR;    // the reference's contact law
};

// Print a failed call's status, message and device error-word bits.
inline void report(int rc, const char* what) {
    gdem_handle* h = engine();
    fprintf(stderr, "%s failed (%d): %s\n", what, rc, h ? gdem_last_error(h) : "");
    gdem_stats s;
    if (h && gdem_stats_get(h, &s) == GDEM_OK && s.error_word) {
        static const char* const names[8] = {"Verlet row over nei_capacity", "wall row over wall_capacity",
                                              "contacts over hist_capacity", "wall contacts over hist_wall_capacity",
                                              "mesh tree stack", "NaN or Inf in a position or velocity",
                                              "active particle outside the cell grid", "bounded wait gave up"};
        fprintf(stderr, "device error word 0x%x:\n", s.error_word);
        for (int b = 0; b < 8; b++)
            if (s.error_word & (1u << b)) fprintf(stderr, "  bit 0x%x: %s\n", 1u << b, names[b]);
    }
}

template <class T>
inline int to_host(const T* d, size_t n, std::vector<T>& h) {
    h.resize(n);
    if (n == 0) return GDEM_OK;
    return cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost) == cudaSuccess ? GDEM_OK : GDEM_ERR_CUDA;
}

// Create the engine from the reference's set-up and import its state.
template <class PS, class Box, class Mesh>
int bind(PS* p, Box* box, Mesh* mesh, int max_nei, const Options& o) {
    const int N = p->N;
    const size_t H = (size_t)N * max_nei;
    gdem_desc d = {};
    d.n_particles = N;
    d.precision = o.precision;
    d.model = o.model;
    d.nei_capacity = max_nei;
    // the engine's maximum: the reference has max_nei slots here too (a case
    // that needs 65..max_nei stops with a capacity bit in the error word)
    d.wall_capacity = 64;
    d.hist_capacity = 64;
    d.hist_wall_capacity = 64;
    d.reorder = 1;
    d.dt = p->dt;
    d.mu = p->mu;
    std::vector<double> g;
    int rc;
    if ((rc = to_host(p->g, 3, g))) return rc;
    for (int c = 0; c < 3; c++) d.g[c] = g[c];
    d.box_min[0] = box->minx; d.box_min[1] = box->miny; d.box_min[2] = box->minz;
    d.box_max[0] = box->maxx; d.box_max[1] = box->maxy; d.box_max[2] = box->maxz;
    d.cell_size = box->dx;
    d.skin = box->skinR;
    d.refresh_thresh = box->refreshThresh;
    gdem_handle* h = nullptr;
    if ((rc = gdem_create(&d, &h))) return rc;
    engine() = h;

    gdem_mesh_arrays m = {};
    m.nVert = mesh->nVert;
    m.nTri = mesh->nTri;
    m.mx = mesh->mx; m.my = mesh->my; m.mz = mesh->mz;
    m.tri_i0 = mesh->tri_i0; m.tri_i1 = mesh->tri_i1; m.tri_i2 = mesh->tri_i2;
    m.tri_e0 = mesh->tri_e0; m.tri_e1 = mesh->tri_e1; m.tri_e2 = mesh->tri_e2;
    m.d = mesh->d;
    if ((rc = gdem_set_mesh_indexed(h, &m))) return rc;

    std::vector<double> x, v, w, r, mass, k, eta, hx, hy, hz, hwx, hwy, hwz;
    std::vector<int> act, nc, ih, ncw, ihw;
    if ((rc = to_host(p->x, 3 * (size_t)N, x)) || (rc = to_host(p->v, 3 * (size_t)N, v)) ||
        (rc = to_host(p->angv, 3 * (size_t)N, w)) || (rc = to_host(p->r, N, r)) || (rc = to_host(p->m, N, mass)) ||
        (rc = to_host(p->k, N, k)) || (rc = to_host(p->etaconst, N, eta)) || (rc = to_host(p->isActive, N, act)) ||
        (rc = to_host(p->numCont, N, nc)) || (rc = to_host(p->indHis, H, ih)) ||
        (rc = to_host(p->numContWall, N, ncw)) || (rc = to_host(p->indHisWall, H, ihw)) ||
        (rc = to_host(p->deltHisx, H, hx)) || (rc = to_host(p->deltHisy, H, hy)) ||
        (rc = to_host(p->deltHisz, H, hz)) || (rc = to_host(p->deltHisxWall, H, hwx)) ||
        (rc = to_host(p->deltHisyWall, H, hwy)) || (rc = to_host(p->deltHiszWall, H, hwz)))
        return rc;
    gdem_particles q = {};
    q.n = N;
    q.x = x.data(); q.v = v.data(); q.angv = w.data();
    q.r = r.data(); q.m = mass.data(); q.k = k.data(); q.etaconst = eta.data();
    q.isActive = act.data();
    q.hist_stride = max_nei;
    q.numCont = nc.data(); q.indHis = ih.data();
    q.deltHisx = hx.data(); q.deltHisy = hy.data(); q.deltHisz = hz.data();
    q.numContWall = ncw.data(); q.indHisWall = ihw.data();
    q.deltHisxWall = hwx.data(); q.deltHisyWall = hwy.data(); q.deltHiszWall = hwz.data();
    return gdem_import_particles(h, &q);
}

// One call of device_dem_verlet_verlet: bind on the first call, then one step.
template <class PS, class Box, class Mesh>
int step(PS* p, Box* box, Mesh* mesh, int max_nei, const Options& o = Options()) {
    if (!engine()) {
        const int rc = bind(p, box, mesh, max_nei, o);
        if (rc) return rc;
    }
    return gdem_step(engine(), 1);
}

// copyFromDevice's SAVE_ON fields, in pId order, into the host struct.
template <class PSh>
int copy_from_device(PSh* ps, int max_nei) {
    gdem_handle* h = engine();
    if (!h) return GDEM_ERR_STATE;
    int rc = gdem_synchronize(h);
    if (rc) return rc;
    gdem_particles q = {};
    q.n = ps->N;
    q.x = ps->x; q.v = ps->v; q.angv = ps->angv;
    q.isActive = ps->isActive;
    q.hist_stride = max_nei;
    q.numCont = ps->numCont; q.indHis = ps->indHis;
    q.deltHisx = ps->deltHisx; q.deltHisy = ps->deltHisy; q.deltHisz = ps->deltHisz;
    q.numContWall = ps->numContWall; q.indHisWall = ps->indHisWall;
    q.deltHisxWall = ps->deltHisxWall; q.deltHisyWall = ps->deltHisyWall; q.deltHiszWall = ps->deltHiszWall;
    return gdem_export_particles(h, &q);
}

// Destroy the engine (the next step call binds again).
inline int release() {
    gdem_handle* h = engine();
    engine() = nullptr;
    return h ? gdem_destroy(h) : GDEM_OK;
}

}  // namespace gdem_shim

#endif  // GDEM_SHIM_CORE_H
