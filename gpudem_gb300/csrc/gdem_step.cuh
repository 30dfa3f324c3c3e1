// The fused step kernel of the GB300 DEM engine, templated on precision
// (FP64 / Mixed) and contact law (linear / Hertz-Mindlin).  One thread per
// particle: particle-particle contacts from the Verlet list, particle-wall
// contacts from the wall list, tangential-history bookkeeping, symplectic
// Euler, the list-refresh test and out-of-bounds marking, in one pass.  Every
// particle accumulates its own force and torque in registers in list order —
// no atomics, deterministic — and writes only its own rows.
//
// It computes one call of device_dem_verlet_verlet (device_dem.cu:1195-1236)
// with the arithmetic of the reference CPU path (cpu_dem.cu):
// particle_collision_verlet :1084, calc_normal_force :953,
// calc_tangential_force :783, update_history :587, wall_collision_verlet :238,
// calc_normal_force_wall :536, calc_tangential_force_wall :636,
// update_history_wall :611, the update loop :1622-1652,
// shouldRefreshNeighborList :1529 and checkOoB :1575.  Instantiated for FP64
// in a translation unit compiled without FMA contraction, the linear law is
// bit-identical to the reference CPU build.
//
// Mixed mode: positions and their integration stay FP64; the pair's relative
// vector is formed in FP64 and then rounded to FP32 (the subtraction cancels,
// the rounding after it does not); contact laws, velocities and spin run in
// FP32; the tangential spring is accumulated with a compensated (Kahan) sum.
#pragma once

#include "gdem_internal.cuh"

namespace gdem {

template <typename R>
struct Vec3 {
    R x, y, z;
};

template <typename R>
__device__ __forceinline__ R sqrt_(R a);
template <>
__device__ __forceinline__ double sqrt_<double>(double a) { return sqrt(a); }
template <>
__device__ __forceinline__ float sqrt_<float>(float a) { return sqrtf(a); }

// Tangential spring update + Coulomb cap (calc_tangential_force,
// cpu_dem.cu:824-891; the wall twin :677-772).  s holds the previous spring on
// entry, the new one on exit; c is its compensation term (mixed mode); ft is
// the force to add.  kt and gt are the tangential stiffness and damping (the
// linear law uses k_i and the normal damping for both).
template <class T>
__device__ __forceinline__ void tangential(typename T::real nx, typename T::real ny, typename T::real nz,
                                           typename T::real fnsq, typename T::real vtx,
                                           typename T::real vty, typename T::real vtz,
                                           typename T::real gt, typename T::real kt,
                                           typename T::real mu, typename T::real dt,
                                           Vec3<typename T::real>& s, Vec3<typename T::real>& c,
                                           Vec3<typename T::real>& ft) {
    using R = typename T::real;
    R dx, dy, dz;
    if (T::mixed) {
        // compensated accumulation of vt*dt
        const R yx = vtx * dt - c.x, yy = vty * dt - c.y, yz = vtz * dt - c.z;
        const R tx = s.x + yx, ty = s.y + yy, tz = s.z + yz;
        c.x = (tx - s.x) - yx;
        c.y = (ty - s.y) - yy;
        c.z = (tz - s.z) - yz;
        dx = tx;
        dy = ty;
        dz = tz;
        const R cdn = c.x * nx + c.y * ny + c.z * nz;
        c.x = c.x - cdn * nx;
        c.y = c.y - cdn * ny;
        c.z = c.z - cdn * nz;
    } else {
        dx = s.x + vtx * dt;
        dy = s.y + vty * dt;
        dz = s.z + vtz * dt;
    }
    const R ddn = dx * nx + dy * ny + dz * nz;
    dx = dx - ddn * nx;
    dy = dy - ddn * ny;
    dz = dz - ddn * nz;
    R tx = -kt * dx, ty = -kt * dy, tz = -kt * dz;
    const R ftsq = tx * tx + ty * ty + tz * tz;
    if (ftsq > (mu * mu) * fnsq) {
        if (ftsq != R(0.)) {
            const R inv = R(1.) / (sqrt_<R>(ftsq) + R(1e-15));
            const R ux = inv * tx, uy = inv * ty, uz = inv * tz;
            const R fnn = sqrt_<R>(fnsq);
            const R sc = mu * fnn;
            tx = sc * ux;
            ty = sc * uy;
            tz = sc * uz;
            const R ik = R(-1.) / kt;
            dx = ik * tx;
            dy = ik * ty;
            dz = ik * tz;
            c.x = R(0.);
            c.y = R(0.);
            c.z = R(0.);
        } else {
            tx = R(0.);
            ty = R(0.);
            tz = R(0.);
        }
    } else {
        tx -= gt * vtx;
        ty -= gt * vty;
        tz -= gt * vtz;
    }
    s.x = dx;
    s.y = dy;
    s.z = dz;
    ft.x = tx;
    ft.y = ty;
    ft.z = tz;
}

// History slot of `key` in row i (linear search, calc_tangential_force
// cpu_dem.cu:795-813), appended when absent; -1 when the row is full.
template <class T>
__device__ __forceinline__ int find_slot(const int* hid, int n, int i, int& nc, int key, int cap,
                                         bool& fresh) {
    for (int q = 0; q < nc; q++)
        if (hid[(size_t)q * n + i] == key) {
            fresh = false;
            return q;
        }
    fresh = true;
    if (nc >= cap) return -1;
    return nc++;
}

template <class T, int MODEL, int WCAP>
__global__ void __launch_bounds__(kBlock) k_step(View<T> v, cudaGraphConditionalHandle cond,
                                                 cudaGraphConditionalHandle /*inner rows: mixed mode only*/,
                                                 int use_cond) {
    using R = typename T::real;
    using V4 = typename T::v4;
    Ctl* ctl = v.ctl;
    const int s = ctl->s, p = ctl->p;
    const int n = v.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const SBank<T> A = v.S[s];
    const SBank<T> B = v.S[s ^ 1];
    const PBank<T> P = v.P[p];
    bool refresh = false;
    unsigned err = 0u;

    if (i < n) {
        const double4_32a pi = A.pos[i];
        const V4 vi = A.vel[i];
        V4 wi = A.rot[i];
        if (wi.w != R(1)) {
            // inactive, or left the box last step (status 2): frozen from now on
            B.pos[i] = pi;
            B.vel[i] = vi;
            wi.w = R(0);
            B.rot[i] = wi;
            if (v.store_forces) {
                v.fx[i] = 0.; v.fy[i] = 0.; v.fz[i] = 0.;
                v.tx[i] = 0.; v.ty[i] = 0.; v.tz[i] = 0.;
            }
        } else {
            const V4 mi = P.mat[i];
            const double xi = pi.x, yi = pi.y, zi = pi.z;
            const R ri = (R)pi.w;
            const R invmi = vi.w;
            const R ki = mi.x, etai = mi.y, sqrtmi = mi.z, invmoi = mi.w;
            const R dt = (R)v.dt;
            // Hertz-Mindlin per-particle materials: both particles of a contact
            // belong to the same scene, so the particle's own values serve
            const bool pm = MODEL == 1 && v.per_particle_mat;
            const R mu = pm ? (R)mi.x : (R)v.mat.mu;
            const R damp_c = pm ? (R)mi.y : (R)v.mat.damp_c;
            R fx = R(0.), fy = R(0.), fz = R(0.);
            R mx = R(0.), my = R(0.), mz = R(0.);

            // ---------------- particle-particle (particle_collision_verlet)
            int nc = P.nc[i];
            unsigned long long touched = 0ull;
            const int nn = v.nnei[i];
            for (int kk = 0; kk < nn; kk++) {
                const int j = v.nei[(size_t)kk * n + i];
                const V4 wj = A.rot[j];
                if (wj.w != R(1)) continue;
                const double4_32a pj = A.pos[j];
                const R dx = (R)image_dx(v, xi - pj.x);
                const R dy = (R)(yi - pj.y);
                const R dz = (R)(zi - pj.z);
                const R distsq = dx * dx + dy * dy + dz * dz;
                const R rj = (R)pj.w;
                const R Rs = ri + rj;
                if (!(distsq < Rs * Rs)) continue;
                const V4 vj = A.vel[j];
                const R dist = sqrt_<R>(distsq);
                const R delMag = Rs - dist;
                const R nx = dx / dist, ny = dy / dist, nz = dz / dist;
                const R vrx = vi.x - vj.x, vry = vi.y - vj.y, vrz = vi.z - vj.z;
                const R vdn = vrx * nx + vry * ny + vrz * nz;
                const R vnx = vdn * nx, vny = vdn * ny, vnz = vdn * nz;
                R fnx, fny, fnz, kt, gt, Rstar = R(0.);
                if (MODEL == 0) {
                    // calc_normal_force (cpu_dem.cu:953-1011)
                    const R delx = -delMag * nx, dely = -delMag * ny, delz = -delMag * nz;
                    const R meff = R(1.) / (invmi + vj.w);
                    const R eta = etai * sqrt_<R>(meff);
                    fnx = -ki * delx - eta * vnx;
                    fny = -ki * dely - eta * vny;
                    fnz = -ki * delz - eta * vnz;
                    kt = ki;
                    gt = eta;
                } else {
                    // Hertz normal, Mindlin tangential stiffness
                    Rstar = ri * rj / (ri + rj);
                    const R mstar = R(1.) / (invmi + vj.w);
                    const R sqrtRd = sqrt_<R>(Rstar * delMag);
                    const R fel = (R)v.mat.kn_c * sqrtRd * delMag;
                    const R gn = damp_c * sqrt_<R>((R)v.mat.sn_c * sqrtRd * mstar);
                    const R fnm = fel - gn * vdn;
                    fnx = fnm * nx;
                    fny = fnm * ny;
                    fnz = fnm * nz;
                    kt = (R)v.mat.kt_c * sqrtRd;
                    gt = damp_c * sqrt_<R>(kt * mstar);
                }
                const R ax_ = ri * wi.x + rj * wj.x;
                const R ay_ = ri * wi.y + rj * wj.y;
                const R az_ = ri * wi.z + rj * wj.z;
                const R crx = ay_ * nz - az_ * ny;
                const R cry = az_ * nx - ax_ * nz;
                const R crz = ax_ * ny - ay_ * nx;
                const R vtx = (vrx - vnx) + crx;
                const R vty = (vry - vny) + cry;
                const R vtz = (vrz - vnz) + crz;
                fx += fnx;
                fy += fny;
                fz += fnz;
                bool fresh;
                const int slot = find_slot<T>(P.hid, n, i, nc, P.pid[j], v.hist_cap, fresh);
                if (slot < 0) {
                    err |= 0x4u;
                    continue;
                }
                const size_t h = (size_t)slot * n + i;
                Vec3<R> sp, cp;
                if (fresh) {
                    P.hid[h] = P.pid[j];
                    sp.x = sp.y = sp.z = R(0.);
                    cp.x = cp.y = cp.z = R(0.);
                } else {
                    sp.x = P.hx[h];
                    sp.y = P.hy[h];
                    sp.z = P.hz[h];
                    if (T::mixed) {
                        cp.x = P.cx[h];
                        cp.y = P.cy[h];
                        cp.z = P.cz[h];
                    } else {
                        cp.x = cp.y = cp.z = R(0.);
                    }
                }
                touched |= 1ull << slot;
                Vec3<R> ft;
                const R fnsq = fnx * fnx + fny * fny + fnz * fnz;
                tangential<T>(nx, ny, nz, fnsq, vtx, vty, vtz, gt, kt, mu, dt, sp, cp, ft);
                fx += ft.x;
                fy += ft.y;
                fz += ft.z;
                const R cx = ny * ft.z - nz * ft.y;
                const R cy = nz * ft.x - nx * ft.z;
                const R cz = nx * ft.y - ny * ft.x;
                mx += ri * cx;
                my += ri * cy;
                mz += ri * cz;
                if (MODEL == 1 && v.mat.mu_roll > 0.) {
                    // rolling resistance, constant torque opposing the relative spin
                    const R rx = wi.x - wj.x, ry = wi.y - wj.y, rz = wi.z - wj.z;
                    const R wn = sqrt_<R>(rx * rx + ry * ry + rz * rz);
                    if (wn > R(0.)) {
                        const R tr = -(R)v.mat.mu_roll * Rstar * sqrt_<R>(fnsq) / wn;
                        mx += tr * rx;
                        my += tr * ry;
                        mz += tr * rz;
                    }
                }
                P.hx[h] = sp.x;
                P.hy[h] = sp.y;
                P.hz[h] = sp.z;
                if (T::mixed) {
                    P.cx[h] = cp.x;
                    P.cy[h] = cp.y;
                    P.cz[h] = cp.z;
                }
            }
            P.nc[i] = surviving(touched, nc);

            // ---------------- particle-wall (wall_collision_verlet)
            int ncw = P.ncw[i];
            unsigned long long wtouched = 0ull;
            const int nw = v.nneiw[i];
            int vore[WCAP];
            int nvore = 0;
            const double rid = pi.w;
            const double rsq = rid * rid;
            for (int kk = 0; kk < nw; kk++) {
                const int t = v.neiw[(size_t)kk * n + i];
                const Feature f = closest_feature(image_x_near(v, xi, v.tri[t].v0[0]), yi, zi, rsq, v.tri[t]);
                if (!(f.dist < rid)) continue;
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
                const R delmag = (R)(rid - f.dist);
                const R nx = (R)f.nx, ny = (R)f.ny, nz = (R)f.nz;
                const R vdn = vi.x * nx + vi.y * ny + vi.z * nz;
                const R vnx = vdn * nx, vny = vdn * ny, vnz = vdn * nz;
                R fnx, fny, fnz, kt, gt;
                if (MODEL == 0) {
                    // calc_normal_force_wall (cpu_dem.cu:536-585): static wall
                    const R delx = -delmag * nx, dely = -delmag * ny, delz = -delmag * nz;
                    const R eta = etai * sqrtmi;
                    fnx = -ki * delx - eta * vnx;
                    fny = -ki * dely - eta * vny;
                    fnz = -ki * delz - eta * vnz;
                    kt = ki;
                    gt = eta;
                } else {
                    const R mstar = R(1.) / invmi;
                    const R sqrtRd = sqrt_<R>(ri * delmag);
                    const R fel = (R)v.mat.kn_c * sqrtRd * delmag;
                    const R gn = damp_c * sqrt_<R>((R)v.mat.sn_c * sqrtRd * mstar);
                    const R fnm = fel - gn * vdn;
                    fnx = fnm * nx;
                    fny = fnm * ny;
                    fnz = fnm * nz;
                    kt = (R)v.mat.kt_c * sqrtRd;
                    gt = damp_c * sqrt_<R>(kt * mstar);
                }
                const R ax_ = ri * wi.x, ay_ = ri * wi.y, az_ = ri * wi.z;
                const R crx = ay_ * nz - az_ * ny;
                const R cry = az_ * nx - ax_ * nz;
                const R crz = ax_ * ny - ay_ * nx;
                const R vtx = (vi.x - vnx) + crx;
                const R vty = (vi.y - vny) + cry;
                const R vtz = (vi.z - vnz) + crz;
                fx += fnx;
                fy += fny;
                fz += fnz;
                bool fresh;
                const int slot = find_slot<T>(P.hwid, n, i, ncw, t, v.histw_cap, fresh);
                if (slot < 0) {
                    err |= 0x8u;
                    continue;
                }
                const size_t h = (size_t)slot * n + i;
                Vec3<R> sp, cp;
                if (fresh) {
                    P.hwid[h] = t;
                    sp.x = sp.y = sp.z = R(0.);
                    cp.x = cp.y = cp.z = R(0.);
                } else {
                    sp.x = P.hwx[h];
                    sp.y = P.hwy[h];
                    sp.z = P.hwz[h];
                    if (T::mixed) {
                        cp.x = P.cwx[h];
                        cp.y = P.cwy[h];
                        cp.z = P.cwz[h];
                    } else {
                        cp.x = cp.y = cp.z = R(0.);
                    }
                }
                wtouched |= 1ull << slot;
                Vec3<R> ft;
                const R fnsq = fnx * fnx + fny * fny + fnz * fnz;
                tangential<T>(nx, ny, nz, fnsq, vtx, vty, vtz, gt, kt, mu, dt, sp, cp, ft);
                fx += ft.x;
                fy += ft.y;
                fz += ft.z;
                const R cx = ny * ft.z - nz * ft.y;
                const R cy = nz * ft.x - nx * ft.z;
                const R cz = nx * ft.y - ny * ft.x;
                mx += ri * cx;
                my += ri * cy;
                mz += ri * cz;
                if (MODEL == 1 && v.mat.mu_roll > 0.) {
                    const R wn = sqrt_<R>(wi.x * wi.x + wi.y * wi.y + wi.z * wi.z);
                    if (wn > R(0.)) {
                        const R tr = -(R)v.mat.mu_roll * ri * sqrt_<R>(fnsq) / wn;
                        mx += tr * wi.x;
                        my += tr * wi.y;
                        mz += tr * wi.z;
                    }
                }
                P.hwx[h] = sp.x;
                P.hwy[h] = sp.y;
                P.hwz[h] = sp.z;
                if (T::mixed) {
                    P.cwx[h] = cp.x;
                    P.cwy[h] = cp.y;
                    P.cwz[h] = cp.z;
                }
            }
            P.ncw[i] = surviving(wtouched, ncw);

            // ---------------- symplectic Euler (cpu_dem.cu:1622-1652)
            const R ax = fx * invmi + (R)v.gx;
            const R ay = fy * invmi + (R)v.gy;
            const R az = fz * invmi + (R)v.gz;
            const R nvx = vi.x + ax * dt, nvy = vi.y + ay * dt, nvz = vi.z + az * dt;
            double nxp, nyp, nzp;
            if (T::mixed) {
                const double ddt = v.dt;
                nxp = xi + (double)nvx * ddt;
                nyp = yi + (double)nvy * ddt;
                nzp = zi + (double)nvz * ddt;
            } else {
                nxp = xi + nvx * dt;
                nyp = yi + nvy * dt;
                nzp = zi + nvz * dt;
            }
            // periodic x: back into the period (a step moves far less than one)
            if (v.per_x) {
                if (nxp >= v.maxx) nxp -= v.Lx;
                else if (nxp < v.minx) nxp += v.Lx;
            }
            const R aax = mx * invmoi, aay = my * invmoi, aaz = mz * invmoi;
            const R nwx = wi.x + aax * dt, nwy = wi.y + aay * dt, nwz = wi.z + aaz * dt;
            // ---------------- refresh test (shouldRefreshNeighborList, cpu_dem.cu:1529):
            // every particle active at the start of the step takes part
            {
                const double4_32a rf = v.ref[i];
                const double ex = image_dx(v, nxp - rf.x), ey = nyp - rf.y, ez = nzp - rf.z;
                const double d2 = ex * ex + ey * ey + ez * ez;
                if (d2 > v.thresh_sq) refresh = true;
            }
            // ---------------- out of bounds (checkOoB, cpu_dem.cu:1575).  The
            // reference CPU loop deactivates after the list rebuild of this
            // step (main.cu:312-316), so a particle leaving the box is marked 2:
            // still in this step's rebuild, inactive from the next step on.
            R status = R(1);
            if ((!v.per_x && (nxp < v.minx || nxp > v.maxx)) || nyp < v.miny || nyp > v.maxy || nzp < v.minz ||
                nzp > v.maxz)
                status = R(2);
            if (!(nxp == nxp && nyp == nyp && nzp == nzp)) {
                err |= 0x20u;
                status = R(2);
            }
            B.pos[i] = make_double4_32a(nxp, nyp, nzp, pi.w);
            V4 nv, nw4;
            nv.x = nvx; nv.y = nvy; nv.z = nvz; nv.w = invmi;
            nw4.x = nwx; nw4.y = nwy; nw4.z = nwz; nw4.w = status;
            B.vel[i] = nv;
            B.rot[i] = nw4;
            if (v.store_forces) {
                v.fx[i] = fx; v.fy[i] = fy; v.fz[i] = fz;
                v.tx[i] = mx; v.ty[i] = my; v.tz[i] = mz;
            }
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

template <class T, int MODEL>
void* step_kernel_for(int wall_cap) {
    if (wall_cap <= 16) return (void*)k_step<T, MODEL, 16>;
    if (wall_cap <= 32) return (void*)k_step<T, MODEL, 32>;
    return (void*)k_step<T, MODEL, 64>;
}

template <class T>
void* step_kernel_any(const View<T>& v) {
    return v.mat.model == 1 ? step_kernel_for<T, 1>(v.wall_cap) : step_kernel_for<T, 0>(v.wall_cap);
}

template <class T>
void launch_step_any(const View<T>& v, cudaStream_t st, cudaGraphConditionalHandle cond, int use_cond) {
    const int g = (v.n + kBlock - 1) / kBlock;
    void* fn = step_kernel_any<T>(v);
    View<T> vv = v;
    cudaGraphConditionalHandle ci = cond;
    void* args[4] = {(void*)&vv, (void*)&cond, (void*)&ci, (void*)&use_cond};
    cudaLaunchKernel(fn, dim3(g), dim3(kBlock), args, 0, st);
}

}  // namespace gdem
