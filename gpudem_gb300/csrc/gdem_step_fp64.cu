// FP64 step kernel of the GB300 DEM engine: contact forces (particle-particle
// from the Verlet list, particle-wall from the wall list), tangential-history
// bookkeeping, symplectic Euler integration, out-of-bounds deactivation and
// the list-refresh test, fused into one pass with one thread per particle.
//
// It computes what one call of device_dem_verlet_verlet does
// (device_dem.cu:1195-1236) with the arithmetic of the reference CPU path
// (cpu_dem.cu): particle_collision_verlet :1084, calc_normal_force :953,
// calc_tangential_force :783, update_history :587, wall_collision_verlet :238,
// calc_normal_force_wall :536, calc_tangential_force_wall :636,
// update_history_wall :611, the update loop :1622-1652, checkOoB :1575 and
// shouldRefreshNeighborList :1529.  Each particle accumulates its own force in
// registers in list order — no atomics, deterministic — and writes only its
// own rows.  Compiled with -fmad=false: FP64 results match the reference CPU
// build (no FMA contraction) bit for bit.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gdem_internal.cuh"

namespace gdem {

namespace {

// Tangential spring update + Coulomb cap shared by particle and wall contacts
// (calc_tangential_force, cpu_dem.cu:824-891; the wall twin :677-772).
// delt holds the previous spring on entry and the new one on exit; ft is the
// tangential force to add.
struct Vec {
    double x, y, z;
};

__device__ __forceinline__ void tangential(double nx, double ny, double nz, double fnx, double fny,
                                           double fnz, double vtx, double vty, double vtz, double eta,
                                           double k, double mu, double dt, Vec& delt, Vec& ft) {
    double dx = delt.x + vtx * dt;
    double dy = delt.y + vty * dt;
    double dz = delt.z + vtz * dt;
    const double ddn = dx * nx + dy * ny + dz * nz;
    dx = dx - ddn * nx;
    dy = dy - ddn * ny;
    dz = dz - ddn * nz;
    double tx = -k * dx, ty = -k * dy, tz = -k * dz;
    const double ftsq = tx * tx + ty * ty + tz * tz;
    const double fnsq = fnx * fnx + fny * fny + fnz * fnz;
    if (ftsq > (mu * mu) * fnsq) {
        if (ftsq != 0.) {
            const double inv = 1. / (sqrt(ftsq) + 1e-15);
            const double ux = inv * tx, uy = inv * ty, uz = inv * tz;
            const double fnn = sqrt(fnsq);
            const double sc = mu * fnn;
            tx = sc * ux;
            ty = sc * uy;
            tz = sc * uz;
            const double ik = -1. / k;
            dx = ik * tx;
            dy = ik * ty;
            dz = ik * tz;
        } else {
            tx = 0.;
            ty = 0.;
            tz = 0.;
        }
    } else {
        tx -= eta * vtx;
        ty -= eta * vty;
        tz -= eta * vtz;
    }
    delt.x = dx;
    delt.y = dy;
    delt.z = dz;
    ft.x = tx;
    ft.y = ty;
    ft.z = tz;
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

}  // namespace

template <int WCAP>
__global__ void __launch_bounds__(kBlock) k_step_fp64(View v, cudaGraphConditionalHandle cond,
                                                      int use_cond) {
    Ctl* ctl = v.ctl;
    const int s = ctl->s, p = ctl->p;
    const int n = v.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const SBank A = v.S[s];
    const SBank B = v.S[s ^ 1];
    const PBank P = v.P[p];
    bool refresh = false;
    unsigned err = 0u;

    if (i < n) {
        if (A.active[i] != 1) {
            // inactive, or left the box last step (2): frozen from now on
            B.x[i] = A.x[i]; B.y[i] = A.y[i]; B.z[i] = A.z[i];
            B.vx[i] = A.vx[i]; B.vy[i] = A.vy[i]; B.vz[i] = A.vz[i];
            B.wx[i] = A.wx[i]; B.wy[i] = A.wy[i]; B.wz[i] = A.wz[i];
            B.active[i] = 0;
            if (v.store_forces) {
                v.fx[i] = 0.; v.fy[i] = 0.; v.fz[i] = 0.;
                v.tx[i] = 0.; v.ty[i] = 0.; v.tz[i] = 0.;
            }
        } else {
            const double xi = A.x[i], yi = A.y[i], zi = A.z[i];
            const double vxi = A.vx[i], vyi = A.vy[i], vzi = A.vz[i];
            const double wxi = A.wx[i], wyi = A.wy[i], wzi = A.wz[i];
            const double ri = P.r[i], ki = P.k[i], etai = P.eta[i], invmi = P.invm[i];
            const double dt = v.dt, mu = v.mu;
            double fx = 0., fy = 0., fz = 0.;
            double mx = 0., my = 0., mz = 0.;

            // ---------------- particle-particle (particle_collision_verlet)
            int nc = P.nc[i];
            unsigned long long touched = 0ull;
            const int nn = v.nnei[i];
            for (int kk = 0; kk < nn; kk++) {
                const int j = v.nei[(size_t)kk * n + i];
                if (A.active[j] != 1) continue;
                const double dx = xi - A.x[j];
                const double dy = yi - A.y[j];
                const double dz = zi - A.z[j];
                const double distsq = dx * dx + dy * dy + dz * dz;
                const double rj = P.r[j];
                const double R = ri + rj;
                if (!(distsq < R * R)) continue;
                const double dist = sqrt(distsq);
                const double delMag = R - dist;
                const double nx = dx / dist, ny = dy / dist, nz = dz / dist;
                // calc_normal_force (cpu_dem.cu:953-1011)
                const double delx = -delMag * nx, dely = -delMag * ny, delz = -delMag * nz;
                const double vrx = vxi - A.vx[j], vry = vyi - A.vy[j], vrz = vzi - A.vz[j];
                const double vdn = vrx * nx + vry * ny + vrz * nz;
                const double vnx = vdn * nx, vny = vdn * ny, vnz = vdn * nz;
                const double meff = 1. / (invmi + P.invm[j]);
                const double eta = etai * sqrt(meff);
                const double fnx = -ki * delx - eta * vnx;
                const double fny = -ki * dely - eta * vny;
                const double fnz = -ki * delz - eta * vnz;
                const double ax_ = ri * wxi + rj * A.wx[j];
                const double ay_ = ri * wyi + rj * A.wy[j];
                const double az_ = ri * wzi + rj * A.wz[j];
                const double crx = ay_ * nz - az_ * ny;
                const double cry = az_ * nx - ax_ * nz;
                const double crz = ax_ * ny - ay_ * nx;
                const double vtx = (vrx - vnx) + crx;
                const double vty = (vry - vny) + cry;
                const double vtz = (vrz - vnz) + crz;
                fx += fnx;
                fy += fny;
                fz += fnz;
                // calc_tangential_force (cpu_dem.cu:783-951): find or append the slot
                const int pj = P.pid[j];
                int slot = -1;
                for (int q = 0; q < nc; q++)
                    if (P.hid[(size_t)q * n + i] == pj) {
                        slot = q;
                        break;
                    }
                Vec delt;
                if (slot < 0) {
                    slot = nc;
                    if (slot >= v.hist_cap) {
                        err |= 0x4u;
                        continue;
                    }
                    nc++;
                    P.hid[(size_t)slot * n + i] = pj;
                    delt.x = 0.;
                    delt.y = 0.;
                    delt.z = 0.;
                } else {
                    delt.x = P.hx[(size_t)slot * n + i];
                    delt.y = P.hy[(size_t)slot * n + i];
                    delt.z = P.hz[(size_t)slot * n + i];
                }
                touched |= 1ull << slot;
                Vec ft;
                tangential(nx, ny, nz, fnx, fny, fnz, vtx, vty, vtz, eta, ki, mu, dt, delt, ft);
                fx += ft.x;
                fy += ft.y;
                fz += ft.z;
                const double cx = ny * ft.z - nz * ft.y;
                const double cy = nz * ft.x - nx * ft.z;
                const double cz = nx * ft.y - ny * ft.x;
                mx += ri * cx;
                my += ri * cy;
                mz += ri * cz;
                P.hx[(size_t)slot * n + i] = delt.x;
                P.hy[(size_t)slot * n + i] = delt.y;
                P.hz[(size_t)slot * n + i] = delt.z;
            }
            P.nc[i] = surviving(touched, nc);

            // ---------------- particle-wall (wall_collision_verlet)
            int ncw = P.ncw[i];
            unsigned long long wtouched = 0ull;
            const int nw = v.nneiw[i];
            int vore[WCAP];
            int nvore = 0;
            const double rsq = P.rsq[i];
            for (int kk = 0; kk < nw; kk++) {
                const int t = v.neiw[(size_t)kk * n + i];
                const Feature f = closest_feature(xi, yi, zi, rsq, v.tri[t]);
                if (!(f.dist < ri)) continue;
                if (f.hit != -1) {
                    // a vertex or edge shared by triangles acts once per step
                    bool dup = false;
                    for (int q = 0; q < nvore; q++)
                        if (vore[q] == f.hit) {
                            dup = true;
                            break;
                        }
                    if (dup) continue;
                    if (nvore < WCAP) vore[nvore++] = f.hit;
                }
                const double delmag = ri - f.dist;
                const double nx = f.nx, ny = f.ny, nz = f.nz;
                // calc_normal_force_wall (cpu_dem.cu:536-585): static wall
                const double delx = -delmag * nx, dely = -delmag * ny, delz = -delmag * nz;
                const double vdn = vxi * nx + vyi * ny + vzi * nz;
                const double vnx = vdn * nx, vny = vdn * ny, vnz = vdn * nz;
                const double eta = etai * P.sqrtm[i];
                const double fnx = -ki * delx - eta * vnx;
                const double fny = -ki * dely - eta * vny;
                const double fnz = -ki * delz - eta * vnz;
                const double ax_ = ri * wxi, ay_ = ri * wyi, az_ = ri * wzi;
                const double crx = ay_ * nz - az_ * ny;
                const double cry = az_ * nx - ax_ * nz;
                const double crz = ax_ * ny - ay_ * nx;
                const double vtx = (vxi - vnx) + crx;
                const double vty = (vyi - vny) + cry;
                const double vtz = (vzi - vnz) + crz;
                fx += fnx;
                fy += fny;
                fz += fnz;
                int slot = -1;
                for (int q = 0; q < ncw; q++)
                    if (P.hwid[(size_t)q * n + i] == t) {
                        slot = q;
                        break;
                    }
                Vec delt;
                if (slot < 0) {
                    slot = ncw;
                    if (slot >= v.histw_cap) {
                        err |= 0x8u;
                        continue;
                    }
                    ncw++;
                    P.hwid[(size_t)slot * n + i] = t;
                    delt.x = 0.;
                    delt.y = 0.;
                    delt.z = 0.;
                } else {
                    delt.x = P.hwx[(size_t)slot * n + i];
                    delt.y = P.hwy[(size_t)slot * n + i];
                    delt.z = P.hwz[(size_t)slot * n + i];
                }
                wtouched |= 1ull << slot;
                Vec ft;
                tangential(nx, ny, nz, fnx, fny, fnz, vtx, vty, vtz, eta, ki, mu, dt, delt, ft);
                fx += ft.x;
                fy += ft.y;
                fz += ft.z;
                const double cx = ny * ft.z - nz * ft.y;
                const double cy = nz * ft.x - nx * ft.z;
                const double cz = nx * ft.y - ny * ft.x;
                mx += ri * cx;
                my += ri * cy;
                mz += ri * cz;
                P.hwx[(size_t)slot * n + i] = delt.x;
                P.hwy[(size_t)slot * n + i] = delt.y;
                P.hwz[(size_t)slot * n + i] = delt.z;
            }
            P.ncw[i] = surviving(wtouched, ncw);

            // ---------------- symplectic Euler (cpu_dem.cu:1622-1652)
            const double ax = fx * invmi + v.gx;
            const double ay = fy * invmi + v.gy;
            const double az = fz * invmi + v.gz;
            const double nvx = vxi + ax * dt, nvy = vyi + ay * dt, nvz = vzi + az * dt;
            const double nxp = xi + nvx * dt, nyp = yi + nvy * dt, nzp = zi + nvz * dt;
            const double invmoi = P.invmoi[i];
            const double aax = mx * invmoi, aay = my * invmoi, aaz = mz * invmoi;
            const double nwx = wxi + aax * dt, nwy = wyi + aay * dt, nwz = wzi + aaz * dt;
            B.x[i] = nxp; B.y[i] = nyp; B.z[i] = nzp;
            B.vx[i] = nvx; B.vy[i] = nvy; B.vz[i] = nvz;
            B.wx[i] = nwx; B.wy[i] = nwy; B.wz[i] = nwz;
            if (v.store_forces) {
                v.fx[i] = fx; v.fy[i] = fy; v.fz[i] = fz;
                v.tx[i] = mx; v.ty[i] = my; v.tz[i] = mz;
            }
            // ---------------- refresh test (shouldRefreshNeighborList, cpu_dem.cu:1529):
            // every particle active at the start of the step takes part
            {
                const double ex = nxp - v.refx[i], ey = nyp - v.refy[i], ez = nzp - v.refz[i];
                const double d2 = ex * ex + ey * ey + ez * ez;
                refresh = d2 > v.thresh_sq;
            }
            // ---------------- out of bounds (checkOoB, cpu_dem.cu:1575).  The
            // reference CPU loop deactivates after the list rebuild of this
            // step (main.cu:312-316), so a particle leaving the box is marked 2:
            // still in this step's rebuild, inactive from the next step on.
            int act = 1;
            if (nxp < v.minx || nxp > v.maxx || nyp < v.miny || nyp > v.maxy || nzp < v.minz ||
                nzp > v.maxz)
                act = 2;
            if (!(nxp == nxp && nyp == nyp && nzp == nzp)) {
                err |= 0x20u;
                act = 2;
            }
            B.active[i] = act;
        }
    }
    if (__any_sync(0xffffffffu, refresh) && (threadIdx.x & 31) == 0) atomicOr(&ctl->refresh, 1u);
    if (err) atomicOr(&ctl->error, err);
    if (last_block(&ctl->done[0])) {
        if (threadIdx.x == 0) {
            ctl->done[0] = 0;
            ctl->s = s ^ 1;
            ctl->steps += 1ull;
            const unsigned r = atomicAdd(&ctl->refresh, 0u);
            if (use_cond) cudaGraphSetConditional(cond, r ? 1u : 0u);
        }
    }
}

void launch_step_fp64(const View& v, cudaStream_t st, cudaGraphConditionalHandle cond, int use_cond) {
    const int g = (v.n + kBlock - 1) / kBlock;
    if (v.wall_cap <= 16)
        k_step_fp64<16><<<g, kBlock, 0, st>>>(v, cond, use_cond);
    else if (v.wall_cap <= 32)
        k_step_fp64<32><<<g, kBlock, 0, st>>>(v, cond, use_cond);
    else
        k_step_fp64<64><<<g, kBlock, 0, st>>>(v, cond, use_cond);
}

void* step_fp64_kernel(int wall_cap) {
    if (wall_cap <= 16) return (void*)k_step_fp64<16>;
    if (wall_cap <= 32) return (void*)k_step_fp64<32>;
    return (void*)k_step_fp64<64>;
}

}  // namespace gdem
