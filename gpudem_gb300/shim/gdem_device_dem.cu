// Reference-side binding of libgdem.so for gpudem's GPU main loop.
//
// Add this file to gpudem's source tree and build it with the reference's
// own flags plus the engine's header, then link the engine:
//
//   nvcc -O3 -DUSE_GPU=1 -arch=sm_103a -I<this repo>/include -I<this repo>/gpudem_gb300/shim \
//        -c gdem_device_dem.cu
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
// read of the state goes through gdem_copy_from_device.  The work itself is
// in gdem_shim_core.h, which reads the structs by member name only.
//
// Capacities.  The reference gives every particle MAX_NEI = 100 slots for its
// Verlet row, its wall row and both contact histories (hardCodedParameters.h:3,
// BVH.cu:277).  The engine keeps 100 Verlet slots but at most 64 for the wall
// row and each history: a particle with 65 to 100 wall candidates or contacts,
// which the reference would still hold, stops the run here with the device
// error word (printed, one GDEM_EW_* bit per capacity) instead of being
// stepped.  Contacts of equal spheres cannot exceed 12, so only unusual
// polydisperse or mesh-dense cases come near 64.
#include <stdio.h>
#include <stdlib.h>

#include "BVH.h"
#include "BoundingBox.h"
#include "ParticleSystem.h"
#include "TriangleMesh.h"
#include "gdem.h"
#include "gdem_shim_core.h"

static void gdem_die_on(int rc, const char* what) {
    if (rc == GDEM_OK) return;
    gdem_shim::report(rc, what);
    exit(1);
}

// Same parameters as device_dem_verlet_verlet (device_dem.h:112); the BVH
// and launch shape are unused: the engine keeps its own mesh tree and launch
// configuration.
void gdem_device_dem_verlet_verlet(ParticleSys<DeviceMemory>* p, BoundingBox* box, TriangleMesh* mesh, BVH* bvh,
                                   int gridSize, int blockSize) {
    (void)bvh;
    (void)gridSize;
    (void)blockSize;
    gdem_die_on(gdem_shim::step(p, box, mesh, MAX_NEI), "gdem step");
}

// Same parameters as copyFromDevice (ParticleSystem.cu:97): fills the
// SAVE_ON fields write_frame_bin and write_single_text read, in pId order.
void gdem_copy_from_device(ParticleSys<DeviceMemory>* d_ps, ParticleSys<HostMemory>* ps) {
    (void)d_ps;
    gdem_die_on(gdem_shim::copy_from_device(ps, MAX_NEI), "gdem copy from device");
}
