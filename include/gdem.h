/*
 * gdem.h — C ABI of the GB300 DEM step engine (libgdem.so).
 *
 * The engine replaces gpudem's per-timestep device path
 *   void device_dem_verlet_verlet(ParticleSys<DeviceMemory>*, BoundingBox*,
 *                                 TriangleMesh*, BVH*, int gridSize, int blockSize)
 * (reference device_dem.h:112, device_dem.cu:1195) and the list builders it
 * calls.  Everything here is plain C: opaque handle, plain pointers and sizes,
 * int status codes, no exceptions across the boundary.  Host arrays use the
 * reference's layouts (ParticleSystem.h member list: xyz-interleaved vectors,
 * MAX_NEI-strided history rows), indexed by particle id (pId) — the index space
 * of the reference CPU path, which never reorders particles.
 *
 * Threading: calls on one handle are not thread-safe.  Work is enqueued on the
 * handle's own CUDA stream; gdem_step returns without waiting.  Every call that
 * returns data to the host waits for the stream first.
 */
#ifndef GDEM_H
#define GDEM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (return value of every call) ---- */
#define GDEM_OK 0
#define GDEM_ERR_ARG 1        /* invalid argument or size */
#define GDEM_ERR_CUDA 2       /* a CUDA runtime call failed (see gdem_last_error) */
#define GDEM_ERR_CAPACITY 3   /* a list or history capacity overflowed on the device */
#define GDEM_ERR_STATE 4      /* call out of order (e.g. step before import) */
#define GDEM_ERR_RANGE 5      /* domain too large for 10-bit Morton cell coordinates */
#define GDEM_ERR_DEVICE 6     /* device error word set (see gdem_stats.error_word) */

/* ---- device error word bits (gdem_stats.error_word) ---- */
#define GDEM_EW_NEI_OVERFLOW 0x1u    /* Verlet list longer than nei_capacity */
#define GDEM_EW_WALL_OVERFLOW 0x2u   /* wall list longer than wall_capacity */
#define GDEM_EW_HIST_OVERFLOW 0x4u   /* more particle contacts than hist_capacity */
#define GDEM_EW_HISTW_OVERFLOW 0x8u  /* more wall contacts than hist_wall_capacity */
#define GDEM_EW_BVH_STACK 0x10u      /* BVH traversal stack exhausted */
#define GDEM_EW_NONFINITE 0x20u      /* NaN or Inf in a position or velocity */
#define GDEM_EW_CELL_RANGE 0x40u     /* active particle outside the cell grid */
#define GDEM_EW_TIMEOUT 0x80u        /* a bounded wait for a bulk copy gave up (results invalid) */

/* ---- modes ---- */
#define GDEM_FP64 0           /* plain FP64, bit-compatible with the reference CPU path */
#define GDEM_MIXED 1          /* FP64 positions/integration, FP32 contact math, Kahan history */
#define GDEM_LINEAR 0         /* linear spring-dashpot + Coulomb (cpu_dem.cu:953, :783) */
#define GDEM_HERTZ_MINDLIN 1  /* Hertz normal + Mindlin tangential + Coulomb (+ rolling) */

typedef struct gdem_handle gdem_handle;

/* Engine creation parameters.  Zero / negative values select the default
 * noted on each field. */
typedef struct gdem_desc {
    int n_particles;        /* particles in the scene (> 0) */
    int precision;          /* GDEM_FP64 (default) or GDEM_MIXED */
    int model;              /* GDEM_LINEAR (default) or GDEM_HERTZ_MINDLIN */
    int nei_capacity;       /* Verlet neighbours per particle, default 64 (reference MAX_NEI=100) */
    int wall_capacity;      /* wall-list triangles per particle, default 32 */
    int hist_capacity;      /* particle contacts kept in history, default 32 */
    int hist_wall_capacity; /* wall contacts kept in history, default 16 */
    int reorder;            /* 1: Morton-reorder particle storage at each list rebuild (default), 0: no */
    int store_forces;       /* 1: keep the last step's force and torque per particle */
    int steps_per_graph;    /* steps unrolled per CUDA graph launch, default 8 */
    double dt;              /* time step (ParticleSysShared::dt) */
    double mu;              /* Coulomb friction coefficient (ParticleSysShared::mu) */
    double g[3];            /* gravity (ParticleSysShared::g) */
    double box_min[3];      /* BoundingBox min/max (BoundingBox.cu:448-478) */
    double box_max[3];
    double cell_size;       /* <= 0: 4 * r_max (BoundingBox.cu:381) in FP64 mode; the list cutoff
                               2 r_max + skin in mixed mode */
    double skin;            /* <= 0: r_max (BoundingBox.cu:386) */
    double refresh_thresh;  /* <= 0: skin / 2 (BoundingBox.cu:387) */
    /* Hertz-Mindlin material (model == GDEM_HERTZ_MINDLIN) */
    double youngs_modulus;
    double poisson_ratio;
    double restitution;
    double rolling_friction;
    int bvh_every_step;     /* 1: rebuild the mesh LBVH (keys, sort, nodes, boxes) in every step, as a
                               moving mesh needs; 0 (default): build it once when the mesh is set */
    /* mixed-precision step kernel (results are the same for every choice):
     * 0 default (warp-cooperative), 1 warp-cooperative, 2 warp-staged, 3 one thread per particle */
    int mixed_kernel;
    int occupancy;          /* resident CTAs per SM its registers are sized for; 0: default (4..6 / 2..3) */
    /* 1: periodic in x.  [box_min[0], box_max[0]) is one period L: a particle
     * leaving through one x face re-enters through the other, and particle pairs
     * and particle-triangle pairs interact through the nearest x image.  The
     * mesh must lie in the period with no triangle wider than L/4 in x; cells
     * are L/floor(L/cell_size) wide in x (at least 3 of them).  No reference
     * counterpart (the reference's box only deactivates what leaves it). */
    int periodic_x;
    /* mixed precision: skin of the inner rows the step kernel scans, the partners
     * of each list row within r_i + r_j + inner_skin, rebuilt from the list rows
     * when a particle has moved half of it (and after every list rebuild).  The
     * contacts and their order are those of the list rows, so results do not
     * change.  0: 0.1 * r_max (at most the skin); < 0: off, the step scans the
     * list rows. */
    double inner_skin;
} gdem_desc;

/* Particle arrays in the reference layout (memberList/ParticleSystemMember_common.def).
 * Row i is the particle with pId i.  Pointers that may be NULL say so. */
typedef struct gdem_particles {
    int n;
    double* x;          /* [3n] positions */
    double* v;          /* [3n] velocities (NULL: zero on import) */
    double* angv;       /* [3n] angular velocities (NULL: zero on import) */
    double* r;          /* [n] radii */
    double* m;          /* [n] masses */
    double* k;          /* [n] normal/tangential stiffness (linear model) */
    double* etaconst;   /* [n] damping constant (ParticleSystem.cu:301) */
    int* isActive;      /* [n] 1 active, 0 out of bounds (NULL: all active on import) */
    /* contact history (NULL: empty on import; skipped on export) */
    int hist_stride;    /* row stride of the history arrays (reference: MAX_NEI = 100) */
    int* numCont;       /* [n] */
    int* indHis;        /* [n*hist_stride] pIds of contacting particles, encounter order */
    double* deltHisx;   /* [n*hist_stride] tangential spring history */
    double* deltHisy;
    double* deltHisz;
    int* numContWall;   /* [n] */
    int* indHisWall;    /* [n*hist_stride] triangle indices */
    double* deltHisxWall;
    double* deltHisyWall;
    double* deltHiszWall;
    /* export only (store_forces = 1): last step's force and torque, [3n] */
    double* f;
    double* mom;
} gdem_particles;

/* Reductions over the active particles (the parity observables). */
typedef struct gdem_stats {
    long long steps;            /* steps taken since import */
    long long rebuilds;         /* Verlet/wall list rebuilds since import */
    long long n_active;
    long long n_nei;            /* sum of Verlet list lengths */
    long long n_wall;           /* sum of wall list lengths */
    long long n_contacts;       /* particle-particle contact history entries (each pair counted twice) */
    long long n_wall_contacts;  /* wall contact history entries */
    double kinetic_energy;      /* sum 0.5 m v.v + 0.5 I w.w */
    double coordination;        /* n_contacts / n_active */
    double packing_fraction;    /* sum of sphere volumes / volume of the particles' bounding box */
    double max_overlap;         /* max over contacts of overlap / (2 r_i) */
    unsigned int error_word;    /* GDEM_EW_* bits */
    int max_nei, max_wall;      /* longest lists seen at the last rebuild */
    long long n_inner;          /* sum of inner row lengths (mixed precision with inner rows) */
    long long inner_builds;     /* inner row rebuilds since import */
    long long n_inner_wall;     /* sum of inner wall row lengths */
} gdem_stats;

/* ---- lifecycle ---- */
int gdem_create(const gdem_desc* desc, gdem_handle** out);
int gdem_destroy(gdem_handle* h);
const char* gdem_last_error(gdem_handle* h);   /* message of the last failing call ("" if none) */

/* Wall mesh from triangle corners in file order (9 doubles per triangle), as an
 * ASCII STL lists them.  file_tri_counts[nfiles] splits the triangles into
 * files; vertices are welded within each file only (TriangleMesh.cu:483-533).
 * NULL/0 means one file.  Replaces load_ascii_stl_double's welding, edge
 * numbering and per-triangle precompute (TriangleMesh.cu:363-752) and the
 * host BVH (BVH.cu:741), which becomes a device LBVH. */
int gdem_set_mesh(gdem_handle* h, const double* tris, int n_tri, const int* file_tri_counts,
                  int nfiles);

/* A mesh the reference's loader has already welded, in its own arrays
 * (TriangleMesh.h:102-170, filled by load_ascii_stl_double,
 * TriangleMesh.cu:363-752).  Vertex ids per triangle ascending, edge ids with
 * nShift already added, d the plane offsets the loader computed. */
typedef struct gdem_mesh_arrays {
    int nVert, nTri;
    const double *mx, *my, *mz;              /* [nVert] vertex coordinates */
    const int *tri_i0, *tri_i1, *tri_i2;     /* [nTri] vertex ids, tri_i0 <= tri_i1 <= tri_i2 */
    const int *tri_e0, *tri_e1, *tri_e2;     /* [nTri] edge ids + nShift */
    const double* d;                         /* [nTri] plane offset -n.x */
} gdem_mesh_arrays;

/* Wall mesh from the reference's loaded TriangleMesh arrays: the same device
 * records, keys and BVH as gdem_set_mesh builds from the STL corners that
 * loader read, without welding again.  This is the call a reference host
 * makes after load_ascii_stl_double (main.cu:99). */
int gdem_set_mesh_indexed(gdem_handle* h, const gdem_mesh_arrays* m);

/* Upload particles (replaces copyToDevice, ParticleSystem.cu:82).  Builds the
 * Verlet and wall lists from the imported state (main.cu:152,199 do this on the
 * host in the reference). */
int gdem_import_particles(gdem_handle* h, const gdem_particles* p);

/* Advance nsteps timesteps (device_dem_verlet_verlet, device_dem.cu:1195, once
 * per step): contacts, integration, out-of-bounds, refresh test and, when a
 * particle moved more than refresh_thresh, the list rebuild — decided on the
 * device, no host synchronisation.  Asynchronous. */
int gdem_step(gdem_handle* h, int nsteps);
int gdem_synchronize(gdem_handle* h);   /* wait; GDEM_ERR_DEVICE if the error word is set */

/* Hertz-Mindlin friction coefficient and restitution per particle (pId
 * order, n values each), in place of the engine-wide mu and restitution: for
 * several independent scenes packed into one engine, each with its own
 * material.  Both particles of a contact must carry the same values.  Call
 * after gdem_import_particles; a later import clears them.  No counterpart in
 * the reference (its material is global, ParticleSysShared::mu). */
int gdem_set_particle_materials(gdem_handle* h, const double* mu, const double* restitution);

/* Download in pId order (replaces copyFromDevice, ParticleSystem.cu:97).
 * Fields left NULL are skipped. */
int gdem_export_particles(gdem_handle* h, gdem_particles* p);

/* Positions only, in pId order (x[3n], the SAVE_ON field write_frame_bin
 * writes every output step, solver_output.cu:259): gathered on the device and
 * copied with one transfer. */
int gdem_export_positions(gdem_handle* h, double* x);

/* gdem_export_positions without waiting: the copy into x (pinned host memory
 * for a true overlap) runs on a copy stream while later steps compute; x is
 * valid after gdem_synchronize.  Two copies may be in flight. */
int gdem_export_positions_async(gdem_handle* h, double* x);

/* ---- particle initialisation on the device ---- */
enum { GDEM_PLACE_RANDOM = 0, GDEM_PLACE_LATTICE = 1 };
enum { GDEM_RADIUS_MONO = 0, GDEM_RADIUS_UNIFORM = 1, GDEM_RADIUS_LOGNORMAL = 2, GDEM_RADIUS_BIDISPERSE = 3 };
/* The reference's "shuffle" inlet (initializeParticles, ParticleSystem.cu:189-340;
 * demSettings.json "inlet"), with polydisperse radii. */
typedef struct gdem_inlet {
    double box_min[3], box_max[3]; /* region of the particle centres (the "shuffle" box) */
    int placement;                 /* GDEM_PLACE_RANDOM: uniform random centres, no two closer than
                                      2 r_max (the reference's rejection sampling, done in parallel);
                                      GDEM_PLACE_LATTICE: jittered cubic sites in random order */
    int radius_dist;               /* GDEM_RADIUS_* */
    double r_a, r_b, r_c, r_d;     /* MONO: r_a.  UNIFORM: [r_a, r_b].  LOGNORMAL: median r_a, sigma of
                                      ln r r_b, clipped to [r_c, r_d].  BIDISPERSE: r_a with probability
                                      r_c, else r_b */
    double density;                /* mass = density * 3.14 * r^3 * 4/3 (main.cu:67) */
    double youngs_modulus;         /* linear law: k = 4/3 (E/2) sqrt(r/2) sqrt(0.05 r) (ParticleSystem.cu:202) */
    double restitution;            /* linear law: etaconst (ParticleSystem.cu:301) */
    double velocity[3];            /* initial velocity: mean ... */
    double velocity_sigma;         /* ... and Gaussian spread per component */
    double gap;                    /* LATTICE: spacing 2 r_max (1 + gap), jitter +-gap r_max / 2 */
    unsigned long long seed;
} gdem_inlet;
/* Place the engine's n_particles particles on the device and import them (as
 * gdem_import_particles would, with no contact history).  GDEM_ERR_RANGE when
 * the region cannot hold them. */
int gdem_init_particles(gdem_handle* h, const gdem_inlet* inlet);

/* ---- output frames and snapshots ---- */
/* Queue the current state's output frame, the file write_frame_bin writes
 * (solver_output.cu:259-316, main.cu:276-286): <dir>/result_%012d.bin with the
 * int32 count of active particles, their float32 positions times
 * length_factor, then their float32 radii times length_factor, in pId order.
 * The frame is built on the device and copied to pinned host memory on a copy
 * stream; a host thread writes the file.  Returns at once: steps launched
 * afterwards run while the frame travels (three frames in flight at most).
 * Replaces copyFromDevice + write_frame_bin at an output step. */
int gdem_frame_write_async(gdem_handle* h, const char* dir, int step, double length_factor);
/* Wait until every queued frame is in its file; reports the first failure. */
int gdem_frames_flush(gdem_handle* h);
/* Checkpoint: the exact state (the precision's own representation, contact
 * histories with every spring term), in pId order, to `path`.  No reference
 * counterpart. */
int gdem_save_snapshot(gdem_handle* h, const char* path);
/* Restart: load a snapshot into an engine created with the same particle
 * count, precision and model, with its mesh set; the run continues bit for
 * bit as if it had not stopped. */
int gdem_load_snapshot(gdem_handle* h, const char* path);
/* Check a snapshot file without a device: its header, its exact length,
 * history counts within the stored capacities, and every history key an index
 * of the stored state (partner particles in [0, n)) or of a mesh of n_tri
 * triangles.  GDEM_OK or GDEM_ERR_ARG.  gdem_load_snapshot runs the same check
 * before it uploads anything. */
int gdem_check_snapshot(const char* path, int n_tri);
int gdem_stats_get(gdem_handle* h, gdem_stats* s);

/* ---- the hot-path stages, callable one at a time ---- */

/* Rebuild Morton order, cell list, Verlet lists and wall lists from the
 * current state now (update_neighborlist + update_neighborlist_wall,
 * BoundingBox.cu:526, BVH.cu:576). */
int gdem_rebuild(gdem_handle* h);

/* Verlet and wall lists in pId space: row p holds the pIds (resp. triangle
 * indices) of the neighbours of particle p in ascending order, like the
 * reference's neiList / neiListWall rows (BoundingBox.cu:579, BVH.cu:622). */
int gdem_export_lists(gdem_handle* h, int stride, int* numNei, int* neiList, int* numNeiWall,
                      int* neiListWall);

/* Morton keys of the particles in pId order, computed as dk_morton_key /
 * update_pList_withSort do (BoundingBox.cu:1007, :680-690). */
int gdem_morton_keys(gdem_handle* h, uint32_t* keys);

/* Cell list of the last rebuild in the layout update_pList_withSort leaves
 * (BoundingBox.cu:664-731): sorted keys, order (pId at each sorted position),
 * pNum/pStart over all cells, pList (sorted positions grouped by cell id).
 * n_cells receives the cell count (BoundingBox::N); pass NULL arrays to query. */
int gdem_export_cells(gdem_handle* h, uint32_t* keys_sorted, int* order, int* pNum, int* pStart,
                      int* pList, int* n_cells);

/* Stable LSB radix sort of n 32-bit keys with index payload 0..n-1 on the
 * device (radixSortUint32, BoundingBox.cu:33; CUB SortPairs, :1235). */
int gdem_sort_keys(const uint32_t* keys, int n, uint32_t* keys_sorted, int* perm);

/* Largest n gdem_sort_keys_noalloc accepts (its fixed device scratch is sized
 * for this many keys: 8.5 MiB). */
#define GDEM_SORT_NOALLOC_MAX_KEYS (1 << 20)

/* The same stable sort as gdem_sort_keys with nothing allocated: d_keys,
 * d_keys_sorted and d_perm are DEVICE pointers on the current device, and the
 * work is enqueued on `stream` (a cudaStream_t; NULL = legacy default stream)
 * without waiting for it.  The scratch is one fixed array per device, looked
 * up on the first call on that device: make that first call before any stream
 * capture begins.  The address is kept with the id of its context; after the
 * context is torn down (cudaDeviceReset) the next call looks it up again, so
 * make that call before any capture too.  Calls on one device must not overlap on the GPU (they share
 * the scratch).  d_keys may equal d_keys_sorted; d_perm must not overlap
 * either.  GDEM_ERR_CAPACITY when n > GDEM_SORT_NOALLOC_MAX_KEYS.
 * No counterpart in the reference: it is for callers that must not allocate
 * device memory while they run (a full device, a fixed memory budget, or a
 * loop that cannot take the device-wide synchronisation of cudaFree). */
int gdem_sort_keys_noalloc(const uint32_t* d_keys, int n, uint32_t* d_keys_sorted, int* d_perm,
                           void* stream);

/* Closest-feature test of m (sphere, triangle) pairs on the device
 * (dist_triangle, cpu_dem.cu:12 / device_dem.cu:12).  out4[4m] = n.xyz, dist;
 * hitAt[m] = -1 face, vertex id, or edge id + nShift; -2 when no contact. */
int gdem_dist_triangle(gdem_handle* h, const double* pos, const double* r, const int* tri, int m,
                       double* out4, int* hitAt);

/* Per-triangle precompute of the current mesh (TriangleMesh.cu:560-667):
 * rec[29*n_tri] doubles per triangle in the order
 *   n.xyz, d, v0.xyz, v1.xyz, v2.xyz, e01.xyz, e02.xyz, e12.xyz,
 *   d00, d01, d11, denom, d00inv, d11inv, d22inv
 * irec[6*n_tri] = tri_i0..2, tri_e0..2; aabb[6*n_tri] = minx,miny,minz,maxx,maxy,maxz;
 * morton[n_tri] sorted centroid keys; sorted_index[n_tri] their permutation. */
int gdem_export_mesh(gdem_handle* h, double* rec, int* irec, double* aabb, uint32_t* morton,
                     int* sorted_index);

/* ---- settings, particle files and walls (the host side of main.cu) ---- */
#define GDEM_INLET_SHUFFLE 0
#define GDEM_INLET_FILE 1
#define GDEM_SETTINGS_MAX_WALLS 16
#define GDEM_SETTINGS_PATH 1024

/* demSettings.json as main.cu reads it (main.cu:44-140; keys in the comments).
 * Numbers the file does not give are NAN where noted. */
typedef struct gdem_settings {
    /* particleTypes.particle0 */
    double radius, restitution, density, mu;  /* radius, CoR, density, mu */
    double youngs_modulus;                    /* YoungModulus; NAN when absent */
    double k_given;                           /* k; NAN when absent */
    /* derived in the reference's operation order */
    double mass;        /* density * 3.14 * r^3 * 4/3 (main.cu:67) */
    double stiffness;   /* 4/3 (E/2) sqrt(r/2) sqrt(0.05 r) (ParticleSystem.cu:202), or k when E is absent */
    double etaconst;    /* -2 ln e sqrt(k / (3.1415^2 + ln^2 e)) (ParticleSystem.cu:301) */
    double dt;          /* 2 PI sqrt(m/k) / dtFactor, snapped to outputTiming / out_step (main.cu:123-129) */
    int out_step;       /* steps per output interval */
    /* inlet */
    int n_particles;    /* numParticle */
    int input_mode;     /* inputMode: GDEM_INLET_SHUFFLE or GDEM_INLET_FILE */
    double inlet_min[3], inlet_max[3];          /* the shuffle box (file mode: NAN; see gdem_read_particle_file) */
    char particle_file[GDEM_SETTINGS_PATH];     /* file mode: the particle file */
    /* walls.filepaths */
    int n_walls;
    char walls[GDEM_SETTINGS_MAX_WALLS][GDEM_SETTINGS_PATH];
    double g[3];        /* gravity.x/y/z */
    /* others */
    int gpu_on, brute_on, seed;                 /* gpuOn; bruteOn (default 0); seed (default 1) */
    double dt_factor, start_time, end_time, output_timing;  /* dtFactor, startTime (default 0), endTime,
                                                               outputTiming */
} gdem_settings;

/* Read demSettings.json (replaces load_json_file and the reads of main.cu:44-140,
 * settings_loader.cu).  Unlike the reference: YoungModulus may be absent (the
 * shipped cases give "k", used as is), bruteOn may be absent (0), and the
 * "file" inlet takes its file name as a string or as {"name": ...} (the
 * reference's string getter accepts only objects, cJSON_d.c:3226-3232).
 * Missing or mistyped keys give GDEM_ERR_ARG and their path in msg (up to
 * msg_len bytes) instead of abort(). */
int gdem_settings_load(const char* path, gdem_settings* s, char* msg, int msg_len);
/* The same from the JSON text itself. */
int gdem_settings_parse(const char* json_text, gdem_settings* s, char* msg, int msg_len);
/* The "file" inlet's particles (ParticleSystem.cu:357-440): a CSV whose header
 * names the columns x, y, z, vx, vy, vz, then exactly n rows.  x[3n] and v[3n]
 * (may be NULL) in file order; box_min/box_max (may be NULL) receive the
 * positions' bounding box, the inlet region of calc_BoundingBoxLimits
 * (BoundingBox.cu:448). */
int gdem_read_particle_file(const char* path, int n, double* x, double* v, double* box_min, double* box_max);
/* Triangles of an ASCII STL file in file order, as load_ascii_stl_double
 * reads them (TriangleMesh.cu:347-386): 9 doubles per triangle into tris (at
 * most cap).  Returns the file's triangle count, -1 if unreadable. */
int gdem_read_stl(const char* path, double* tris, int cap);

/* ---- measurement ---- */

/* The CUDA stream (cudaStream_t) every call of this handle enqueues on, for
 * recording timing events around gdem_step. */
int gdem_get_stream(gdem_handle* h, void** stream);

/* Time the step kernel alone: `iters` launches (rounded up to a multiple of
 * 4) in groups of 4 back to back, each group bracketed by CUDA events on the
 * handle's stream and followed by the device-gated list rebuild.  A rebuild
 * that a step requests therefore runs up to 3 steps late: the lists stay
 * valid while no particle moves more than skin/2 in 3 steps.  avg_ms receives
 * the mean step-kernel duration.  Advances the simulation by the launches. */
int gdem_profile_step(gdem_handle* h, int iters, float* avg_ms);

#ifdef __cplusplus
}
#endif
#endif /* GDEM_H */
