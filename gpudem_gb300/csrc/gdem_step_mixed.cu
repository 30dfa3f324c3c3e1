// Mixed-precision step kernel of the GB300 DEM engine.
//
// Same step as the FP64 kernel (gdem_step.cuh: contacts from the Verlet and
// wall lists, tangential history, symplectic Euler, refresh test, out-of-box
// marking), arranged so that GB300's scarce FP64 pipe is used a few times per
// particle instead of per neighbour:
//  * every particle's position is kept twice: the FP64 master (pos, integrated
//    in FP64 and read by the list rebuild) and an unevaluated float pair
//    x = hi + lo (posh/posl, ~48-bit significand).  A pair's relative vector
//    is (hi_i - hi_j) + (lo_i - lo_j) in FP32: the first difference is exact
//    for nearby particles, so the vector is formed at FP64 accuracy before it
//    is rounded, as the overlap r_i + r_j - |x_ij| needs;
//  * the pair is advanced with an error-free FP32 sum each step and re-split
//    from the FP64 master at every list rebuild;
//  * wall contacts use FP32 triangle records with the first corner as a float
//    pair, and the plane distance taken relative to that corner;
//  * contact laws, velocities and spin are FP32; the tangential spring is a
//    compensated (Kahan) sum;
//  * the refresh test and the out-of-box test use the float pairs.
// Compiled with multiply-add contraction on.
#include <stdlib.h>

#include "gdem_step.cuh"

namespace gdem {

namespace {

struct FeatureF {
    float nx, ny, nz, dist;
    int hit;
};

// Closest feature of triangle T to the sphere centre (ph + pl) within radius^2
// rsq: the classification of dist_triangle (cpu_dem.cu:12-205) in FP32 on the
// corner-relative vector.
__device__ __forceinline__ FeatureF closest_feature_f(float3 ph, float3 pl, float rsq, const TriRecF& T) {
    FeatureF res;
    res.nx = res.ny = res.nz = 0.f;
    res.dist = 1.e10f;
    res.hit = -2;
    const float ax = (ph.x - T.v0h[0]) + (pl.x - T.v0l[0]);
    const float ay = (ph.y - T.v0h[1]) + (pl.y - T.v0l[1]);
    const float az = (ph.z - T.v0h[2]) + (pl.z - T.v0l[2]);
    const float dist = T.n[0] * ax + T.n[1] * ay + T.n[2] * az;
    if (dist * dist > rsq) return res;
    const float d20 = ax * T.e01[0] + ay * T.e01[1] + az * T.e01[2];
    const float d21 = ax * T.e02[0] + ay * T.e02[1] + az * T.e02[2];
    const float v = (T.d11 * d20 - T.d01 * d21) * T.denom;
    const float w = (T.d00 * d21 - T.d01 * d20) * T.denom;
    const float u = 1.0f - v - w;
    if (u > 0.f && v > 0.f && w > 0.f) {
        const float sign = dist < 0.f ? -1.f : 1.f;
        res.nx = sign * T.n[0];
        res.ny = sign * T.n[1];
        res.nz = sign * T.n[2];
        res.dist = sign * dist;
        res.hit = -1;
        return res;
    }
    float rx, ry, rz;  // centre minus the closest point
    int hit;
    if (v <= 0.f && w <= 0.f) {
        rx = ax; ry = ay; rz = az;
        hit = T.i0;
    } else if (u <= 0.f && w <= 0.f) {
        rx = ax - T.e01[0]; ry = ay - T.e01[1]; rz = az - T.e01[2];
        hit = T.i1;
    } else if (u <= 0.f && v <= 0.f) {
        rx = ax - T.e02[0]; ry = ay - T.e02[1]; rz = az - T.e02[2];
        hit = T.i2;
    } else if (u <= 0.f) {
        const float bx = ax - T.e01[0], by = ay - T.e01[1], bz = az - T.e01[2];
        float t = (bx * T.e12[0] + by * T.e12[1] + bz * T.e12[2]) * T.d22inv;
        t = fmaxf(0.f, fminf(1.f, t));
        rx = bx - t * T.e12[0]; ry = by - t * T.e12[1]; rz = bz - t * T.e12[2];
        hit = T.e1;
    } else if (v <= 0.f) {
        float t = d21 * T.d11inv;
        t = fmaxf(0.f, fminf(1.f, t));
        rx = ax - t * T.e02[0]; ry = ay - t * T.e02[1]; rz = az - t * T.e02[2];
        hit = T.e2;
    } else {
        float t = d20 * T.d00inv;
        t = fmaxf(0.f, fminf(1.f, t));
        rx = ax - t * T.e01[0]; ry = ay - t * T.e01[1]; rz = az - t * T.e01[2];
        hit = T.e0;
    }
    const float dsq = rx * rx + ry * ry + rz * rz;
    if (dsq < rsq) {
        const float inv = rsqrtf(dsq);
        res.dist = dsq * inv;
        res.nx = rx * inv;
        res.ny = ry * inv;
        res.nz = rz * inv;
    }
    res.hit = hit;
    return res;
}

// (hi, lo) += d with an error-free sum (Knuth's TwoSum, then a fast
// renormalisation).  Intrinsic adds: no multiply may be contracted into them.
__device__ __forceinline__ void pair_add(float& hi, float& lo, float d) {
    const float s = __fadd_rn(hi, d);
    const float bb = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(d, bb));
    const float l = __fadd_rn(lo, e);
    hi = __fadd_rn(s, l);
    lo = __fsub_rn(l, __fsub_rn(hi, s));
}

}  // namespace

template <int MODEL, int WCAP, int MINB>
__global__ void __launch_bounds__(kBlock, MINB) k_step_mixed(View<Mixed> v, cudaGraphConditionalHandle cond,
                                                            int use_cond) {
    using T = Mixed;
    using R = float;
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
        float4 wi = A.rot[i];
        const float4 hi = A.posh[i];
        float4 li = A.posl[i];
        const float4 vi = A.vel[i];
        if (wi.w != 1.f) {
            // inactive, or left the box last step (status 2): frozen from now on
            B.pos[i] = A.pos[i];
            B.posh[i] = hi;
            li.w = 0.f;
            B.posl[i] = li;
            B.vel[i] = vi;
            B.vell[i] = A.vell[i];
            B.rotl[i] = A.rotl[i];
            wi.w = 0.f;
            B.rot[i] = wi;
            if (v.store_forces) {
                v.fx[i] = 0.; v.fy[i] = 0.; v.fz[i] = 0.;
                v.tx[i] = 0.; v.ty[i] = 0.; v.tz[i] = 0.;
            }
        } else {
            const float4 mi = P.mat[i];
            const R ri = hi.w;
            const R invmi = vi.w;
            const R ki = mi.x, etai = mi.y, sqrtmi = mi.z, invmoi = mi.w;
            const R dt = (R)v.dt, mu = (R)v.mat.mu;
            R fx = 0.f, fy = 0.f, fz = 0.f;
            R mx = 0.f, my = 0.f, mz = 0.f;

            // ---------------- particle-particle
            int nc = P.nc[i];
            unsigned long long touched = 0ull;
            const int nn = v.nnei[i];
            for (int kk = 0; kk < nn; kk++) {
                const int j = v.nei[(size_t)kk * n + i];
                const float4 lj = A.posl[j];
                if (lj.w != 1.f) continue;
                const float4 hj = A.posh[j];
                const R dx = (hi.x - hj.x) + (li.x - lj.x);
                const R dy = (hi.y - hj.y) + (li.y - lj.y);
                const R dz = (hi.z - hj.z) + (li.z - lj.z);
                const R distsq = dx * dx + dy * dy + dz * dz;
                const R rj = hj.w;
                const R Rs = ri + rj;
                if (!(distsq < Rs * Rs)) continue;
                const float4 vj = A.vel[j];
                const float4 wj = A.rot[j];
                const R dist = sqrtf(distsq);
                const R inv = 1.f / dist;
                const R delMag = Rs - dist;
                const R nx = dx * inv, ny = dy * inv, nz = dz * inv;
                const R vrx = vi.x - vj.x, vry = vi.y - vj.y, vrz = vi.z - vj.z;
                const R vdn = vrx * nx + vry * ny + vrz * nz;
                const R vnx = vdn * nx, vny = vdn * ny, vnz = vdn * nz;
                R fnx, fny, fnz, kt, gt, Rstar = 0.f;
                if (MODEL == 0) {
                    const R meff = 1.f / (invmi + vj.w);
                    const R eta = etai * sqrtf(meff);
                    const R fel = ki * delMag;
                    fnx = fel * nx - eta * vnx;
                    fny = fel * ny - eta * vny;
                    fnz = fel * nz - eta * vnz;
                    kt = ki;
                    gt = eta;
                } else {
                    Rstar = ri * rj / Rs;
                    const R mstar = 1.f / (invmi + vj.w);
                    const R sqrtRd = sqrtf(Rstar * delMag);
                    const R fel = (R)v.mat.kn_c * sqrtRd * delMag;
                    const R gn = (R)v.mat.damp_c * sqrtf((R)v.mat.sn_c * sqrtRd * mstar);
                    const R fnm = fel - gn * vdn;
                    fnx = fnm * nx;
                    fny = fnm * ny;
                    fnz = fnm * nz;
                    kt = (R)v.mat.kt_c * sqrtRd;
                    gt = (R)v.mat.damp_c * sqrtf(kt * mstar);
                }
                const R ax_ = ri * wi.x + rj * wj.x;
                const R ay_ = ri * wi.y + rj * wj.y;
                const R az_ = ri * wi.z + rj * wj.z;
                const R vtx = (vrx - vnx) + (ay_ * nz - az_ * ny);
                const R vty = (vry - vny) + (az_ * nx - ax_ * nz);
                const R vtz = (vrz - vnz) + (ax_ * ny - ay_ * nx);
                fx += fnx;
                fy += fny;
                fz += fnz;
                const int pj = P.pid[j];
                bool fresh;
                const int slot = find_slot<T>(P.hid, n, i, nc, pj, v.hist_cap, fresh);
                if (slot < 0) {
                    err |= 0x4u;
                    continue;
                }
                const size_t h = (size_t)slot * n + i;
                Vec3<R> sp, cp;
                if (fresh) {
                    P.hid[h] = pj;
                    sp.x = sp.y = sp.z = 0.f;
                    cp.x = cp.y = cp.z = 0.f;
                } else {
                    sp.x = P.hx[h]; sp.y = P.hy[h]; sp.z = P.hz[h];
                    cp.x = P.cx[h]; cp.y = P.cy[h]; cp.z = P.cz[h];
                }
                touched |= 1ull << slot;
                Vec3<R> ft;
                const R fnsq = fnx * fnx + fny * fny + fnz * fnz;
                tangential<T>(nx, ny, nz, fnsq, vtx, vty, vtz, gt, kt, mu, dt, sp, cp, ft);
                fx += ft.x;
                fy += ft.y;
                fz += ft.z;
                mx += ri * (ny * ft.z - nz * ft.y);
                my += ri * (nz * ft.x - nx * ft.z);
                mz += ri * (nx * ft.y - ny * ft.x);
                if (MODEL == 1 && v.mat.mu_roll > 0.) {
                    const R rx = wi.x - wj.x, ry = wi.y - wj.y, rz = wi.z - wj.z;
                    const R wn2 = rx * rx + ry * ry + rz * rz;
                    if (wn2 > 0.f) {
                        const R tr = -(R)v.mat.mu_roll * Rstar * sqrtf(fnsq) * rsqrtf(wn2);
                        mx += tr * rx;
                        my += tr * ry;
                        mz += tr * rz;
                    }
                }
                P.hx[h] = sp.x; P.hy[h] = sp.y; P.hz[h] = sp.z;
                P.cx[h] = cp.x; P.cy[h] = cp.y; P.cz[h] = cp.z;
            }
            P.nc[i] = surviving(touched, nc);

            // ---------------- particle-wall
            int ncw = P.ncw[i];
            unsigned long long wtouched = 0ull;
            const int nw = v.nneiw[i];
            int vore[WCAP];
            int nvore = 0;
            const float3 ph = make_float3(hi.x, hi.y, hi.z), pl = make_float3(li.x, li.y, li.z);
            const R rsq = ri * ri;
            for (int kk = 0; kk < nw; kk++) {
                const int t = v.neiw[(size_t)kk * n + i];
                const FeatureF f = closest_feature_f(ph, pl, rsq, v.trif[t]);
                if (!(f.dist < ri)) continue;
                if (f.hit != -1) {
                    bool dup = false;
                    for (int q = 0; q < nvore; q++)
                        if (vore[q] == f.hit) {
                            dup = true;
                            break;
                        }
                    if (dup) continue;
                    if (nvore < WCAP) vore[nvore++] = f.hit;
                }
                const R delmag = ri - f.dist;
                const R nx = f.nx, ny = f.ny, nz = f.nz;
                const R vdn = vi.x * nx + vi.y * ny + vi.z * nz;
                const R vnx = vdn * nx, vny = vdn * ny, vnz = vdn * nz;
                R fnx, fny, fnz, kt, gt;
                if (MODEL == 0) {
                    const R eta = etai * sqrtmi;
                    const R fel = ki * delmag;
                    fnx = fel * nx - eta * vnx;
                    fny = fel * ny - eta * vny;
                    fnz = fel * nz - eta * vnz;
                    kt = ki;
                    gt = eta;
                } else {
                    const R mstar = 1.f / invmi;
                    const R sqrtRd = sqrtf(ri * delmag);
                    const R fel = (R)v.mat.kn_c * sqrtRd * delmag;
                    const R gn = (R)v.mat.damp_c * sqrtf((R)v.mat.sn_c * sqrtRd * mstar);
                    const R fnm = fel - gn * vdn;
                    fnx = fnm * nx;
                    fny = fnm * ny;
                    fnz = fnm * nz;
                    kt = (R)v.mat.kt_c * sqrtRd;
                    gt = (R)v.mat.damp_c * sqrtf(kt * mstar);
                }
                const R ax_ = ri * wi.x, ay_ = ri * wi.y, az_ = ri * wi.z;
                const R vtx = (vi.x - vnx) + (ay_ * nz - az_ * ny);
                const R vty = (vi.y - vny) + (az_ * nx - ax_ * nz);
                const R vtz = (vi.z - vnz) + (ax_ * ny - ay_ * nx);
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
                    sp.x = sp.y = sp.z = 0.f;
                    cp.x = cp.y = cp.z = 0.f;
                } else {
                    sp.x = P.hwx[h]; sp.y = P.hwy[h]; sp.z = P.hwz[h];
                    cp.x = P.cwx[h]; cp.y = P.cwy[h]; cp.z = P.cwz[h];
                }
                wtouched |= 1ull << slot;
                Vec3<R> ft;
                const R fnsq = fnx * fnx + fny * fny + fnz * fnz;
                tangential<T>(nx, ny, nz, fnsq, vtx, vty, vtz, gt, kt, mu, dt, sp, cp, ft);
                fx += ft.x;
                fy += ft.y;
                fz += ft.z;
                mx += ri * (ny * ft.z - nz * ft.y);
                my += ri * (nz * ft.x - nx * ft.z);
                mz += ri * (nx * ft.y - ny * ft.x);
                if (MODEL == 1 && v.mat.mu_roll > 0.) {
                    const R wn2 = wi.x * wi.x + wi.y * wi.y + wi.z * wi.z;
                    if (wn2 > 0.f) {
                        const R tr = -(R)v.mat.mu_roll * ri * sqrtf(fnsq) * rsqrtf(wn2);
                        mx += tr * wi.x;
                        my += tr * wi.y;
                        mz += tr * wi.z;
                    }
                }
                P.hwx[h] = sp.x; P.hwy[h] = sp.y; P.hwz[h] = sp.z;
                P.cwx[h] = cp.x; P.cwy[h] = cp.y; P.cwz[h] = cp.z;
            }
            P.ncw[i] = surviving(wtouched, ncw);

            // ---------------- symplectic Euler.  Velocity and spin are float
            // pairs, so their many small increments do not round away.
            float4 vl = A.vell[i], wl = A.rotl[i];
            float nvx = vi.x, nvy = vi.y, nvz = vi.z;
            pair_add(nvx, vl.x, (fx * invmi + (R)v.gx) * dt);
            pair_add(nvy, vl.y, (fy * invmi + (R)v.gy) * dt);
            pair_add(nvz, vl.z, (fz * invmi + (R)v.gz) * dt);
            // displacement v*dt as a float pair (the product's rounding error by FMA)
            const R sx = nvx * dt, sy = nvy * dt, sz = nvz * dt;
            const R ex_ = fmaf(nvx, dt, -sx) + vl.x * dt;
            const R ey_ = fmaf(nvy, dt, -sy) + vl.y * dt;
            const R ez_ = fmaf(nvz, dt, -sz) + vl.z * dt;
            // FP64 master
            const double4_32a pi = A.pos[i];
            B.pos[i] = make_double4_32a(pi.x + ((double)sx + (double)ex_), pi.y + ((double)sy + (double)ey_),
                                        pi.z + ((double)sz + (double)ez_), pi.w);
            // float pair
            float4 nh = hi, nl = li;
            pair_add(nh.x, nl.x, sx);
            pair_add(nh.y, nl.y, sy);
            pair_add(nh.z, nl.z, sz);
            nl.x += ex_;
            nl.y += ey_;
            nl.z += ez_;
            float nwx = wi.x, nwy = wi.y, nwz = wi.z;
            pair_add(nwx, wl.x, mx * invmoi * dt);
            pair_add(nwy, wl.y, my * invmoi * dt);
            pair_add(nwz, wl.z, mz * invmoi * dt);
            B.vell[i] = vl;
            B.rotl[i] = wl;
            // refresh test against the reference position of the last rebuild
            {
                const float4 rh = v.refh[i], rl = v.refl[i];
                const R ex = (nh.x - rh.x) + (nl.x - rl.x);
                const R ey = (nh.y - rh.y) + (nl.y - rl.y);
                const R ez = (nh.z - rh.z) + (nl.z - rl.z);
                refresh = (double)(ex * ex + ey * ey + ez * ez) > v.thresh_sq;
            }
            // out of bounds (the box rounded outwards to FP32)
            R status = 1.f;
            if (nh.x < v.boxf[0] || nh.x > v.boxf[3] || nh.y < v.boxf[1] || nh.y > v.boxf[4] ||
                nh.z < v.boxf[2] || nh.z > v.boxf[5])
                status = 2.f;
            if (!(nvx == nvx && nvy == nvy && nvz == nvz)) {
                err |= 0x20u;
                status = 2.f;
            }
            nl.w = status;
            B.posh[i] = nh;
            B.posl[i] = nl;
            B.vel[i] = make_float4(nvx, nvy, nvz, invmi);
            B.rot[i] = make_float4(nwx, nwy, nwz, status);
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

namespace {
// MINB: resident blocks per SM the register allocation is sized for (3, the
// default: more warps in flight, a few spills; 2: no spills).  GDEM_MIXED_MINB
// picks one.
template <int MODEL, int MINB>
void* mixed_kernel_minb(int wall_cap) {
    if (wall_cap <= 16) return (void*)k_step_mixed<MODEL, 16, MINB>;
    if (wall_cap <= 32) return (void*)k_step_mixed<MODEL, 32, MINB>;
    return (void*)k_step_mixed<MODEL, 64, MINB>;
}
template <int MODEL>
void* mixed_kernel_for(int wall_cap) {
    static const int minb = [] {
        const char* e = getenv("GDEM_MIXED_MINB");
        return e ? atoi(e) : 3;
    }();
    return minb == 3 ? mixed_kernel_minb<MODEL, 3>(wall_cap) : mixed_kernel_minb<MODEL, 2>(wall_cap);
}
}  // namespace

void* step_kernel(const View<Mixed>& v) {
    return v.mat.model == 1 ? mixed_kernel_for<1>(v.wall_cap) : mixed_kernel_for<0>(v.wall_cap);
}

void launch_step(const View<Mixed>& v, cudaStream_t st, cudaGraphConditionalHandle cond, int use_cond) {
    const int g = (v.n + kBlock - 1) / kBlock;
    View<Mixed> vv = v;
    void* args[3] = {(void*)&vv, (void*)&cond, (void*)&use_cond};
    cudaLaunchKernel(step_kernel(v), dim3(g), dim3(kBlock), args, 0, st);
}

}  // namespace gdem
