/*
 * Test-infrastructure harness around the UNMODIFIED gpudem CPU step path.
 *
 * This file is compiled together with the reference's own sources
 * (cpu_dem.cu, BoundingBox.cu, BVH.cu, TriangleMesh.cu, ParticleSystem.cu,
 * cJSON_d.c) by oracle/build_ref.sh, into oracle/_ref/librefharness.so.  It is
 * only used to generate and check golden vectors (tests/golden/make_golden.py)
 * and to validate the CPU restatement in oracle/gdem_oracle.cpp.  It is never
 * part of the product and never runs on the GPU.
 *
 * The harness owns what the reference's main.cu owns (main.cu:30-245): it
 * fills ParticleSys<HostMemory> directly from caller arrays (skipping the
 * O(N^2) placement of ParticleSystem.cu:219-285), writes the mesh to an ASCII
 * STL file and loads it with load_ascii_stl_double (TriangleMesh.cu:363), builds
 * the bounding box (BoundingBox.cu:364), the initial Verlet lists
 * (BoundingBox.cu:526), the BVH (BVH.cu:628,741) and wall lists (BVH.cu:576),
 * then steps with cpu_dem_verlet_verlet + checkOoB exactly like the CPU loop of
 * main.cu:302-316.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
#include "ParticleSystem.h"
#include "BoundingBox.h"
#include "TriangleMesh.h"
#include "BVH.h"
#include "cpu_dem.h"
#include "cJSON_d.h"

struct RefHandle {
    ParticleSys<HostMemory> ps;
    ParticleSys<HostMemory> tmp;
    BoundingBox box;
    TriangleMesh mesh;
    BVH bvh;
    int step;
    int rebuilds;
    int nTri;
};

static void fill_particles(ParticleSys<HostMemory>* p, int N, const double* x, const double* v,
                           const double* w, const double* r, const double* m, const double* k,
                           const double* eta) {
    /* zero every array first so unused list slots are deterministic */
#define MEMBER(type, name, Np, SAVE_FLAG) memset(p->name, 0, sizeof(type) * (size_t)(Np));
    {
#include "memberList/ParticleSystemMember_common.def"
    }
#undef MEMBER
    p->steps = 0;
    p->length_factor = 1.0;
    p->mass_factor = 1.0;
    p->time_factor = 1.0;
    for (int i = 0; i < N; i++) {
        for (int d = 0; d < 3; d++) {
            p->x[i * 3 + d] = x[i * 3 + d];
            p->v[i * 3 + d] = v ? v[i * 3 + d] : 0.;
            p->angv[i * 3 + d] = w ? w[i * 3 + d] : 0.;
            p->anga[i * 3 + d] = 0.;
        }
        /* same derived quantities, same operation order as ParticleSystem.cu:294-335 */
        p->r[i] = r[i];
        p->rsq[i] = p->r[i] * p->r[i];
        p->invr[i] = 1. / p->r[i];
        p->k[i] = k[i];
        p->m[i] = m[i];
        p->sqrtm[i] = sqrt(m[i]);
        p->invm[i] = 1. / m[i];
        p->etaconst[i] = eta[i];
        p->cellId[i] = -1;
        p->isActive[i] = 1;
        p->numCont[i] = 0;
        p->numContWall[i] = 0;
        p->moi[i] = 2. / 5. * p->m[i] * p->rsq[i];
        p->invmoi[i] = 1. / p->moi[i];
        p->pId[i] = i;
        for (int j = 0; j < MAX_NEI; j++) {
            p->indHis[i * MAX_NEI + j] = -1;
            p->indHisWall[i * MAX_NEI + j] = -1;
            p->indHisWallNow[i * MAX_NEI + j] = -1;
            p->isContact[i * MAX_NEI + j] = -1;
            p->isContactWall[i * MAX_NEI + j] = -1;
        }
    }
}

static int write_stl(const char* path, int nTri, const double* tri) {
    FILE* fp = fopen(path, "w");
    if (!fp) return -1;
    fprintf(fp, "solid harness\n");
    for (int t = 0; t < nTri; t++) {
        fprintf(fp, "facet normal 0 0 0\nouter loop\n");
        for (int c = 0; c < 3; c++)
            fprintf(fp, "vertex %.17g %.17g %.17g\n", tri[t * 9 + c * 3 + 0], tri[t * 9 + c * 3 + 1],
                    tri[t * 9 + c * 3 + 2]);
        fprintf(fp, "endloop\nendfacet\n");
    }
    fprintf(fp, "endsolid harness\n");
    fclose(fp);
    return 0;
}

extern "C" {

/* mu, dt and g are scene scalars; inlet_min/max enter the box limits the way
 * calc_BoundingBoxLimits (BoundingBox.cu:448) reads them; skinR/refreshThresh
 * <= 0 keep the reference defaults (skin = r_max, threshold = r_max/2). */
void* rh_create(int N, const double* x, const double* v, const double* w, const double* r,
                const double* m, const double* k, const double* eta, double mu, double dt,
                const double* g, int nTri, const double* tri, const double* inlet_min,
                const double* inlet_max, double skinR, double refreshThresh) {
    RefHandle* h = new RefHandle();
    memset(&h->box, 0, sizeof(h->box));
    memset(&h->mesh, 0, sizeof(h->mesh));
    memset(&h->bvh, 0, sizeof(h->bvh));
    h->ps.N = N;
    h->tmp.N = N;
    h->ps.mu = mu;
    allocate(&h->ps);
    allocate(&h->tmp);
    fill_particles(&h->ps, N, x, v, w, r, m, k, eta);
    fill_particles(&h->tmp, N, x, v, w, r, m, k, eta);
    h->ps.g[0] = g[0];
    h->ps.g[1] = g[1];
    h->ps.g[2] = g[2];
    h->ps.dt = dt;
    h->ps.mu = mu;

    char path[] = "/tmp/gdem_ref_meshXXXXXX";
    int fd = mkstemp(path);
    if (fd < 0) return NULL;
    close(fd);
    write_stl(path, nTri, tri);
    cJSON* arr = cJSON_CreateArray();
    cJSON_AddItemToArray(arr, cJSON_CreateString(path));
    load_ascii_stl_double(arr, &h->mesh);
    cJSON_Delete(arr);
    unlink(path);
    h->nTri = nTri;

    cJSON* inlet = cJSON_CreateObject();
    cJSON_AddNumberToObject(inlet, "minx", inlet_min[0]);
    cJSON_AddNumberToObject(inlet, "miny", inlet_min[1]);
    cJSON_AddNumberToObject(inlet, "minz", inlet_min[2]);
    cJSON_AddNumberToObject(inlet, "maxx", inlet_max[0]);
    cJSON_AddNumberToObject(inlet, "maxy", inlet_max[1]);
    cJSON_AddNumberToObject(inlet, "maxz", inlet_max[2]);
    initialize_BoundingBox(&h->ps, &h->box, &h->mesh, inlet, 0);
    cJSON_Delete(inlet);
    if (skinR > 0.) {
        h->box.skinR = skinR;
        h->box.refreshThresh = refreshThresh;
        h->box.refreshThreshSq = refreshThresh * refreshThresh;
    }

    update_neighborlist(&h->ps, &h->tmp, &h->box);
    initializeBVH(&h->bvh, h->mesh.nTri, 0);
    buildBVH(&h->bvh, &h->mesh);
    update_neighborlist_wall(&h->ps, &h->mesh, &h->bvh, h->box.skinR);
    h->step = 0;
    h->rebuilds = 0;
    return h;
}

/* one iteration of the CPU loop of main.cu:302-316; returns the number of
 * neighbour-list rebuilds observed (refx changes only on a rebuild) */
int rh_step(void* hv, int nsteps) {
    RefHandle* h = (RefHandle*)hv;
    int N = h->ps.N;
    double* oldref = (double*)malloc(sizeof(double) * 3 * (size_t)N);
    int nreb = 0;
    for (int s = 0; s < nsteps; s++) {
        for (int i = 0; i < N; i++) {
            oldref[i * 3 + 0] = h->ps.refx[i];
            oldref[i * 3 + 1] = h->ps.refy[i];
            oldref[i * 3 + 2] = h->ps.refz[i];
        }
        h->step += 1;
        cpu_dem_verlet_verlet(&h->ps, &h->tmp, &h->box, &h->mesh, &h->bvh, h->step);
        checkOoB(&h->ps, &h->tmp, &h->box);
        int changed = 0;
        for (int i = 0; i < N && !changed; i++)
            changed = (oldref[i * 3 + 0] != h->ps.refx[i]) || (oldref[i * 3 + 1] != h->ps.refy[i]) ||
                      (oldref[i * 3 + 2] != h->ps.refz[i]);
        nreb += changed;
    }
    h->rebuilds += nreb;
    free(oldref);
    return nreb;
}

void rh_set_active(void* hv, const int* active) {
    RefHandle* h = (RefHandle*)hv;
    for (int i = 0; i < h->ps.N; i++) h->ps.isActive[i] = active[i];
}

/* copy a named particle array out; returns element count or -1 */
long rh_get_particle(void* hv, const char* name, void* out) {
    RefHandle* h = (RefHandle*)hv;
    ParticleSys<HostMemory>* p = &h->ps;
    int N = p->N;
#define MEMBER(type, nm, Np, SAVE_FLAG)                              \
    if (strcmp(name, #nm) == 0) {                                    \
        memcpy(out, p->nm, sizeof(type) * (size_t)(Np));             \
        return (long)(Np);                                           \
    }
#include "memberList/ParticleSystemMember_common.def"
#undef MEMBER
    return -1;
}

/* box scalars: min[3], max[3], dx[3], invd[3], skinR, refreshThresh, refreshThreshSq, range[3]
 * and sizes: sizex, sizey, sizez, N */
void rh_get_box(void* hv, double* d, int* iv) {
    RefHandle* h = (RefHandle*)hv;
    BoundingBox* b = &h->box;
    double vals[18] = {b->minx, b->miny, b->minz, b->maxx, b->maxy, b->maxz, b->dx, b->dy, b->dz,
                       b->invdx, b->invdy, b->invdz, b->skinR, b->refreshThresh, b->refreshThreshSq,
                       b->rangex, b->rangey, b->rangez};
    memcpy(d, vals, sizeof(vals));
    iv[0] = b->sizex;
    iv[1] = b->sizey;
    iv[2] = b->sizez;
    iv[3] = b->N;
}

/* mesh arrays by name (per-triangle doubles/ints, vertex arrays, sorted index, morton keys) */
long rh_get_mesh(void* hv, const char* name, void* out) {
    RefHandle* h = (RefHandle*)hv;
    TriangleMesh* m = &h->mesh;
    int Nt = m->nTri, Nv = m->nVert;
#define TD(nm)                                                      \
    if (strcmp(name, #nm) == 0) {                                   \
        memcpy(out, m->nm, sizeof(double) * (size_t)Nt);            \
        return Nt;                                                  \
    }
#define TI(nm)                                                      \
    if (strcmp(name, #nm) == 0) {                                   \
        memcpy(out, m->nm, sizeof(int) * (size_t)Nt);               \
        return Nt;                                                  \
    }
    TD(nx) TD(ny) TD(nz) TD(d) TD(e01x) TD(e01y) TD(e01z) TD(e02x) TD(e02y) TD(e02z) TD(e12x) TD(e12y)
    TD(e12z) TD(d00) TD(d00inv) TD(d01) TD(d11) TD(d11inv) TD(d22) TD(d22inv) TD(denom) TD(minx)
    TD(maxx) TD(miny) TD(maxy) TD(minz) TD(maxz) TD(cx) TD(cy) TD(cz)
    TI(tri_i0) TI(tri_i1) TI(tri_i2) TI(tri_e0) TI(tri_e1) TI(tri_e2) TI(sortedIndex)
#undef TD
#undef TI
    if (strcmp(name, "mortonKey") == 0) {
        memcpy(out, m->mortonKey, sizeof(uint32_t) * (size_t)Nt);
        return Nt;
    }
    if (strcmp(name, "mx") == 0) { memcpy(out, m->mx, sizeof(double) * (size_t)Nv); return Nv; }
    if (strcmp(name, "my") == 0) { memcpy(out, m->my, sizeof(double) * (size_t)Nv); return Nv; }
    if (strcmp(name, "mz") == 0) { memcpy(out, m->mz, sizeof(double) * (size_t)Nv); return Nv; }
    if (strcmp(name, "nShift") == 0) { *(int*)out = m->nShift; return 1; }
    if (strcmp(name, "gbox") == 0) {
        double g[6] = {m->gminx, m->gminy, m->gminz, m->gmaxx, m->gmaxy, m->gmaxz};
        memcpy(out, g, sizeof(g));
        return 6;
    }
    return -1;
}

long rh_get_bvh(void* hv, const char* name, void* out) {
    RefHandle* h = (RefHandle*)hv;
    BVH* b = &h->bvh;
    int n = b->nodeCount;
    if (strcmp(name, "minx") == 0) { memcpy(out, b->minx, sizeof(double) * n); return n; }
    if (strcmp(name, "miny") == 0) { memcpy(out, b->miny, sizeof(double) * n); return n; }
    if (strcmp(name, "minz") == 0) { memcpy(out, b->minz, sizeof(double) * n); return n; }
    if (strcmp(name, "maxx") == 0) { memcpy(out, b->maxx, sizeof(double) * n); return n; }
    if (strcmp(name, "maxy") == 0) { memcpy(out, b->maxy, sizeof(double) * n); return n; }
    if (strcmp(name, "maxz") == 0) { memcpy(out, b->maxz, sizeof(double) * n); return n; }
    if (strcmp(name, "left") == 0) { memcpy(out, b->left, sizeof(int) * n); return n; }
    if (strcmp(name, "right") == 0) { memcpy(out, b->right, sizeof(int) * n); return n; }
    if (strcmp(name, "tri") == 0) { memcpy(out, b->tri, sizeof(int) * n); return n; }
    return -1;
}

/* Rebuild Verlet + wall lists now from the current state (BoundingBox.cu:526, BVH.cu:576). */
void rh_rebuild_lists(void* hv) {
    RefHandle* h = (RefHandle*)hv;
    update_neighborlist(&h->ps, &h->tmp, &h->box);
    update_neighborlist_wall(&h->ps, &h->mesh, &h->bvh, h->box.skinR);
}

/* Canonical cell CSR (BoundingBox.cu:839): pNum/pStart over all cells, pList. */
void rh_update_plist(void* hv, int* pNum, int* pStart, int* pList, int* cellId, int* cellx) {
    RefHandle* h = (RefHandle*)hv;
    update_pList(&h->ps, &h->box);
    memcpy(pNum, h->box.pNum, sizeof(int) * (size_t)h->box.N);
    memcpy(pStart, h->box.pStart, sizeof(int) * (size_t)h->box.N);
    memcpy(pList, h->box.pList, sizeof(int) * (size_t)h->ps.N);
    memcpy(cellId, h->ps.cellId, sizeof(int) * (size_t)h->ps.N);
    memcpy(cellx, h->ps.cellx, sizeof(int) * 3 * (size_t)h->ps.N);
}

/* Morton sort + particle reorder + cell CSR (BoundingBox.cu:664).  Reorders the
 * handle's particles.  Outputs the sorted keys, the permutation (new -> old),
 * pNum/pStart over all cells, pList, and the reordered pId. */
void rh_update_plist_withsort(void* hv, unsigned int* keys_sorted, int* order, int* pNum,
                              int* pStart, int* pList, int* pId) {
    RefHandle* h = (RefHandle*)hv;
    update_pList_withSort(&h->ps, &h->tmp, &h->box);
    int N = h->ps.N;
    memcpy(keys_sorted, h->ps.mortonKey, sizeof(uint32_t) * (size_t)N);
    memcpy(order, h->ps.mortonOrder, sizeof(int) * (size_t)N);
    memcpy(pNum, h->box.pNum, sizeof(int) * (size_t)h->box.N);
    memcpy(pStart, h->box.pStart, sizeof(int) * (size_t)h->box.N);
    memcpy(pList, h->box.pList, sizeof(int) * (size_t)N);
    memcpy(pId, h->ps.pId, sizeof(int) * (size_t)N);
}

/* radixSortUint32 (BoundingBox.cu:33) on caller keys with index payload 0..N-1 */
void rh_radix_sort(int N, const unsigned int* keys, unsigned int* keys_out, int* perm_out) {
    uint32_t* k = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(N > 0 ? N : 1));
    uint32_t* kw = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(N > 0 ? N : 1));
    int* ix = (int*)malloc(sizeof(int) * (size_t)(N > 0 ? N : 1));
    int* iw = (int*)malloc(sizeof(int) * (size_t)(N > 0 ? N : 1));
    for (int i = 0; i < N; i++) {
        k[i] = keys[i];
        ix[i] = i;
    }
    uint32_t* kp = k;
    int* ip = ix;
    radixSortUint32(&kp, &ip, N, kw, iw);
    memcpy(keys_out, kp, sizeof(uint32_t) * (size_t)N);
    memcpy(perm_out, ip, sizeof(int) * (size_t)N);
    free(k);
    free(kw);
    free(ix);
    free(iw);
}

unsigned int rh_morton3d(unsigned int x, unsigned int y, unsigned int z) { return morton3D(x, y, z); }

/* dist_triangle (cpu_dem.cu:12) for particle i vs triangle j: n[3], dist, hitAt */
void rh_dist_triangle(void* hv, int i, int j, double* out4, int* hitAt) {
    RefHandle* h = (RefHandle*)hv;
    TriangleContactCache tc = dist_triangle(&h->ps, i, &h->mesh, j);
    out4[0] = tc.n.x;
    out4[1] = tc.n.y;
    out4[2] = tc.n.z;
    out4[3] = tc.dist;
    *hitAt = (tc.dist < 1e9) ? tc.hitAt : -2;
}

/* The reference's own initializeParticles (ParticleSystem.cu:189-340) on a
 * "shuffle" inlet of N particles of radius r in [lo, hi], with the mass
 * main.cu:67 computes from the density (its expression, restated here since
 * main.cu is not part of the harness) and the Young's modulus and
 * restitution it passes.  Out: x[3N] and per particle m, k, etaconst, moi,
 * invmoi, sqrtm, invm. */
int rh_init_particles(int N, double r, double density, double E, double res, const double* lo, const double* hi,
                      double* x, double* m, double* k, double* eta, double* moi, double* invmoi, double* sqrtm,
                      double* invm) {
    ParticleSys<HostMemory> ps;
    memset(&ps, 0, sizeof(ps));
    ps.N = N;
    allocate(&ps);
    const double mass = density * 3.14 * r * r * r * 4. / 3.;
    cJSON* inlet = cJSON_CreateObject();
    cJSON_AddStringToObject(inlet, "inputMode", "shuffle");
    cJSON* sh = cJSON_CreateObject();
    cJSON_AddNumberToObject(sh, "minx", lo[0]);
    cJSON_AddNumberToObject(sh, "miny", lo[1]);
    cJSON_AddNumberToObject(sh, "minz", lo[2]);
    cJSON_AddNumberToObject(sh, "maxx", hi[0]);
    cJSON_AddNumberToObject(sh, "maxy", hi[1]);
    cJSON_AddNumberToObject(sh, "maxz", hi[2]);
    cJSON_AddItemToObject(inlet, "shuffle", sh);
    initializeParticles(&ps, inlet, r, mass, E, res);
    cJSON_Delete(inlet);
    for (int i = 0; i < N; i++) {
        for (int d = 0; d < 3; d++) x[3 * i + d] = ps.x[3 * i + d];
        m[i] = ps.m[i];
        k[i] = ps.k[i];
        eta[i] = ps.etaconst[i];
        moi[i] = ps.moi[i];
        invmoi[i] = ps.invmoi[i];
        sqrtm[i] = ps.sqrtm[i];
        invm[i] = ps.invm[i];
    }
    deallocate(&ps);
    return 0;
}

int rh_step_count(void* hv) { return ((RefHandle*)hv)->step; }
int rh_num_tri(void* hv) { return ((RefHandle*)hv)->mesh.nTri; }
int rh_node_count(void* hv) { return ((RefHandle*)hv)->bvh.nodeCount; }

void rh_destroy(void* hv) {
    RefHandle* h = (RefHandle*)hv;
    deallocate(&h->ps);
    deallocate(&h->tmp);
    free_TriangleMesh(&h->mesh, 0);
    free_BoundingBox(&h->box, 0);
    free_BVH(&h->bvh, 0);
    delete h;
}

}  // extern "C"
