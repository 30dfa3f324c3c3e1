// Mixed-precision step kernel of the GB300 DEM engine.
//
// Same step as the FP64 kernel (gdem_step.cuh: contacts from the Verlet and
// wall lists, tangential history, symplectic Euler, refresh test, out-of-box
// marking), arranged so that GB300's scarce FP64 pipe is used a few times per
// particle instead of per neighbour:
//  * every position is an unevaluated float pair x = hi + lo (posh/posl,
//    about 48 significant bits), advanced with an error-free FP32 sum each
//    step; the list rebuild reads hi + lo in FP64, where it is exact.  A
//    pair's relative vector is (hi_i - hi_j) + (lo_i - lo_j) in FP32: the
//    first difference is exact for nearby particles, so the vector is formed
//    at FP64 accuracy before it is rounded, as the overlap r_i + r_j - |x_ij|
//    needs;
//  * wall contacts use FP32 triangle records with the first corner as a float
//    pair, and the plane distance taken relative to that corner;
//  * contact laws, velocities and spin are FP32; the tangential spring is a
//    compensated (Kahan) sum;
//  * the refresh test and the out-of-box test use the high parts;
//  * no FP64 arithmetic at all: the scalars arrive pre-rounded to FP32.
// Compiled with multiply-add contraction on.
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

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

// End of a step kernel: refresh vote, error bits, and in the last CTA the
// bank flip, the step count and the graph's rebuild condition.
__device__ __forceinline__ void step_epilogue(Ctl* ctl, int s, bool refresh, unsigned err,
                                              cudaGraphConditionalHandle cond, int use_cond) {
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

// State of one particle at the start of a step (bank s), however it was
// brought in: straight from HBM, or staged in shared memory by bulk copies.
struct Own {
    float4 wi, hi, li, vi, vl, wl, rh;
    int nn, nw, nc, ncw;
};

// One particle's step: contacts, history, integration, refresh and
// out-of-box tests.  Writes bank s^1 and the history.
template <int MODEL, int WCAP>
__device__ __forceinline__ void step_one(const View<Mixed>& v, const SBank<Mixed>& A, const SBank<Mixed>& B,
                                         const PBank<Mixed>& P, int i, Own o, bool& refresh, unsigned& err,
                                         const int* nei_s = nullptr, int nei_s_rows = 0) {
    using T = Mixed;
    using R = float;
    const int n = v.n;
    const float4* __restrict__ Aposh = A.posh;
    const float4* __restrict__ Aposl = A.posl;
    const float4* __restrict__ Avel = A.vel;
    const float4* __restrict__ Arot = A.rot;
    const int* __restrict__ nei = v.nei;
    const int* __restrict__ neiw = v.neiw;
    const int* __restrict__ pid = P.pid;
    float4 wi = o.wi;
    const float4 hi = o.hi;
    float4 li = o.li;
    const float4 vi = o.vi;
    float4 vl = o.vl;
    float4 wl = o.wl;
    if (wi.w != 1.f) {
        // inactive, or left the box last step (status 2): frozen from now on
        B.posh[i] = hi;
        li.w = 0.f;
        B.posl[i] = li;
        B.vel[i] = vi;
        B.vell[i] = vl;
        B.rotl[i] = wl;
        wi.w = 0.f;
        B.rot[i] = wi;
        if (v.store_forces) {
            v.fx[i] = 0.; v.fy[i] = 0.; v.fz[i] = 0.;
            v.tx[i] = 0.; v.ty[i] = 0.; v.tz[i] = 0.;
        }
    } else {
        const float4 rh = o.rh;
        const int nn = o.nn;
        const int nw = o.nw;
        int nc = o.nc;
        int ncw = o.ncw;
        const R ri = hi.w;
        const R invmi = vi.w;
        R ki = 0.f, etai = 0.f, sqrtmi = 0.f, invmoi;
        if (MODEL == 0) {
            const float4 mi = __ldg(&P.mat[i]);
            ki = mi.x; etai = mi.y; sqrtmi = mi.z; invmoi = mi.w;
        } else {
            invmoi = 2.5f * invmi / (ri * ri);  // 1 / (2/5 m r^2)
        }
        const R dt = v.dtf, mu = v.muf;
        R fx = 0.f, fy = 0.f, fz = 0.f;
        R mx = 0.f, my = 0.f, mz = 0.f;

        // ---------------- particle-particle.  The row is read four
        // entries at a time so their gathers are in flight together; the
        // contacts among them are then handled one by one in row order.
        unsigned long long touched = 0ull;
        for (int k0 = 0; k0 < nn; k0 += 4) {
            int jj[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int k = k0 + q;
                jj[q] = k < nn ? (k < nei_s_rows ? nei_s[k * 32] : __ldg(&nei[(size_t)k * n + i])) : -1;
            }
            float4 hj[4], lj[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (jj[q] >= 0) {
                    hj[q] = __ldg(&Aposh[jj[q]]);
                    lj[q] = __ldg(&Aposl[jj[q]]);
                }
            }
            unsigned hit = 0u;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (jj[q] < 0 || lj[q].w != 1.f) continue;
                const R dx = (hi.x - hj[q].x) + (li.x - lj[q].x);
                const R dy = (hi.y - hj[q].y) + (li.y - lj[q].y);
                const R dz = (hi.z - hj[q].z) + (li.z - lj[q].z);
                const R Rs = ri + hj[q].w;
                if (dx * dx + dy * dy + dz * dz < Rs * Rs) hit |= 1u << q;
            }
            while (hit) {
                const int q = __ffs(hit) - 1;
                hit &= hit - 1u;
                const int k = k0 + q;
                const int j = k < nei_s_rows ? nei_s[k * 32] : __ldg(&nei[(size_t)k * n + i]);
                const float4 hjq = __ldg(&Aposh[j]), ljq = __ldg(&Aposl[j]);
                const R dx = (hi.x - hjq.x) + (li.x - ljq.x);
                const R dy = (hi.y - hjq.y) + (li.y - ljq.y);
                const R dz = (hi.z - hjq.z) + (li.z - ljq.z);
                const R distsq = dx * dx + dy * dy + dz * dz;
                const R rj = hjq.w;
                const R Rs = ri + rj;
                const float4 vj = __ldg(&Avel[j]);
                const float4 wj = __ldg(&Arot[j]);
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
                    const R fel = v.kn_cf * sqrtRd * delMag;
                    const R gn = v.damp_cf * sqrtf(v.sn_cf * sqrtRd * mstar);
                    const R fnm = fel - gn * vdn;
                    fnx = fnm * nx;
                    fny = fnm * ny;
                    fnz = fnm * nz;
                    kt = v.kt_cf * sqrtRd;
                    gt = v.damp_cf * sqrtf(kt * mstar);
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
                const int pj = __ldg(&pid[j]);
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
                if (MODEL == 1 && v.mu_rollf > 0.f) {
                    const R rx = wi.x - wj.x, ry = wi.y - wj.y, rz = wi.z - wj.z;
                    const R wn2 = rx * rx + ry * ry + rz * rz;
                    if (wn2 > 0.f) {
                        const R tr = -v.mu_rollf * Rstar * sqrtf(fnsq) * rsqrtf(wn2);
                        mx += tr * rx;
                        my += tr * ry;
                        mz += tr * rz;
                    }
                }
                P.hx[h] = sp.x; P.hy[h] = sp.y; P.hz[h] = sp.z;
                P.cx[h] = cp.x; P.cy[h] = cp.y; P.cz[h] = cp.z;
            }
        }
        P.nc[i] = surviving(touched, nc);

        // ---------------- particle-wall
        unsigned long long wtouched = 0ull;
        int vore[WCAP];
        int nvore = 0;
        const float3 ph = make_float3(hi.x, hi.y, hi.z), pl = make_float3(li.x, li.y, li.z);
        const R rsq = ri * ri;
        for (int kk = 0; kk < nw; kk++) {
            const int t = __ldg(&neiw[(size_t)kk * n + i]);
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
                const R fel = v.kn_cf * sqrtRd * delmag;
                const R gn = v.damp_cf * sqrtf(v.sn_cf * sqrtRd * mstar);
                const R fnm = fel - gn * vdn;
                fnx = fnm * nx;
                fny = fnm * ny;
                fnz = fnm * nz;
                kt = v.kt_cf * sqrtRd;
                gt = v.damp_cf * sqrtf(kt * mstar);
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
            if (MODEL == 1 && v.mu_rollf > 0.f) {
                const R wn2 = wi.x * wi.x + wi.y * wi.y + wi.z * wi.z;
                if (wn2 > 0.f) {
                    const R tr = -v.mu_rollf * ri * sqrtf(fnsq) * rsqrtf(wn2);
                    mx += tr * wi.x;
                    my += tr * wi.y;
                    mz += tr * wi.z;
                }
            }
            P.hwx[h] = sp.x; P.hwy[h] = sp.y; P.hwz[h] = sp.z;
            P.cwx[h] = cp.x; P.cwy[h] = cp.y; P.cwz[h] = cp.z;
        }
        P.ncw[i] = surviving(wtouched, ncw);

        // ---------------- symplectic Euler.  Position, velocity and spin
        // are float pairs, so their many small increments do not round away.
        float nvx = vi.x, nvy = vi.y, nvz = vi.z;
        pair_add(nvx, vl.x, (fx * invmi + v.gxf) * dt);
        pair_add(nvy, vl.y, (fy * invmi + v.gyf) * dt);
        pair_add(nvz, vl.z, (fz * invmi + v.gzf) * dt);
        // displacement v*dt as a float pair (the product's rounding error by FMA)
        const R sx = nvx * dt, sy = nvy * dt, sz = nvz * dt;
        const R ex_ = fmaf(nvx, dt, -sx) + vl.x * dt;
        const R ey_ = fmaf(nvy, dt, -sy) + vl.y * dt;
        const R ez_ = fmaf(nvz, dt, -sz) + vl.z * dt;
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
        // refresh test against the position of the last rebuild, on the
        // high parts: it only decides when the lists are rebuilt, and the
        // threshold leaves a margin of skin/2 to the list cutoff
        {
            const R ex = nh.x - rh.x, ey = nh.y - rh.y, ez = nh.z - rh.z;
            refresh = ex * ex + ey * ey + ez * ez > v.thresh_sqf;
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

// One thread per particle, state loaded straight from HBM.
template <int MODEL, int WCAP, int MINB>
__global__ void __launch_bounds__(kBlock, MINB) k_step_mixed(View<Mixed> v, cudaGraphConditionalHandle cond,
                                                            int use_cond) {
    Ctl* ctl = v.ctl;
    const int s = ctl->s, p = ctl->p;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const SBank<Mixed> A = v.S[s];
    const SBank<Mixed> B = v.S[s ^ 1];
    const PBank<Mixed> P = v.P[p];
    bool refresh = false;
    unsigned err = 0u;
    if (i < v.n) {
        Own o;
        o.wi = __ldg(&A.rot[i]);
        o.hi = __ldg(&A.posh[i]);
        o.li = __ldg(&A.posl[i]);
        o.vi = __ldg(&A.vel[i]);
        o.vl = __ldg(&A.vell[i]);
        o.wl = __ldg(&A.rotl[i]);
        o.rh = __ldg(&v.refh[i]);
        o.nn = __ldg(&v.nnei[i]);
        o.nw = __ldg(&v.nneiw[i]);
        o.nc = P.nc[i];
        o.ncw = P.ncw[i];
        step_one<MODEL, WCAP>(v, A, B, P, i, o, refresh, err);
    }
    step_epilogue(ctl, s, refresh, err, cond, use_cond);
}

// ---------------------------------------------------------------- TMA-staged
// Persistent variant: each CTA walks tiles of kBlock consecutive particles.
// The per-particle arrays of a tile are contiguous, so one thread brings a
// whole tile in with bulk copies (cp.async.bulk, completion counted on an
// mbarrier) while the CTA works on the previous tile out of the other buffer.
// The first Verlet-list rows of the next tile are prefetched into L2 the
// same way.  Every wait on an mbarrier gives up after kSpinLimit tries and
// sets GDEM_EW_TIMEOUT.
constexpr int kNeiPrefetchRows = 8;
constexpr unsigned kSpinLimit = 1u << 22;

struct __align__(16) Stage {
    float4 posh[kBlock], posl[kBlock], vel[kBlock], rot[kBlock], vell[kBlock], rotl[kBlock], refh[kBlock];
    int nnei[kBlock], nneiw[kBlock], nc[kBlock], ncw[kBlock];
};
constexpr int kStageBytes = (int)sizeof(Stage);

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0u;
}
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
    for (unsigned k = 0; k < kSpinLimit; k++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, unsigned bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// Issue the bulk copies of tile `t` into `st` (one thread).  The tail tile's
// int arrays are copied in whole 16-byte units: every array is allocated in
// 256-byte units, so the rounded copy stays inside its allocation.
__device__ __forceinline__ void issue_tile(const View<Mixed>& v, const SBank<Mixed>& A, const PBank<Mixed>& P,
                                           int t, Stage* st, unsigned long long* bar) {
    const int base = t * kBlock;
    const int cnt = min(kBlock, v.n - base);
    const unsigned b16 = 16u * (unsigned)cnt;
    const unsigned b4 = 4u * (unsigned)((cnt + 3) & ~3);
    mbar_expect_tx(bar, 7u * b16 + 4u * b4);
    bulk_g2s(st->posh, A.posh + base, b16, bar);
    bulk_g2s(st->posl, A.posl + base, b16, bar);
    bulk_g2s(st->vel, A.vel + base, b16, bar);
    bulk_g2s(st->rot, A.rot + base, b16, bar);
    bulk_g2s(st->vell, A.vell + base, b16, bar);
    bulk_g2s(st->rotl, A.rotl + base, b16, bar);
    bulk_g2s(st->refh, v.refh + base, b16, bar);
    bulk_g2s(st->nnei, v.nnei + base, b4, bar);
    bulk_g2s(st->nneiw, v.nneiw + base, b4, bar);
    bulk_g2s(st->nc, P.nc + base, b4, bar);
    bulk_g2s(st->ncw, P.ncw + base, b4, bar);
    // Verlet rows k*n + [base, base+cnt) of the tile, rounded out to 16 bytes
    // (inside the list's allocation: row 0 starts 1 KiB-aligned, the last row
    // ends inside the final 256-byte unit)
    const int rows = min(kNeiPrefetchRows, v.nei_cap);
    for (int k = 0; k < rows; k++) {
        const uintptr_t a = (uintptr_t)(v.nei + (size_t)k * v.n + base);
        const uintptr_t lo = a & ~(uintptr_t)15, hi = (a + 4u * (unsigned)cnt + 15u) & ~(uintptr_t)15;
        bulk_prefetch_l2((const void*)lo, (unsigned)(hi - lo));
    }
}

template <int MODEL, int WCAP>
__global__ void __launch_bounds__(kBlock, 2) k_step_mixed_tma(View<Mixed> v, cudaGraphConditionalHandle cond,
                                                             int use_cond) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Stage* stage = reinterpret_cast<Stage*>(smem_raw);
    __shared__ __align__(8) unsigned long long full[2];
    Ctl* ctl = v.ctl;
    const int s = ctl->s, p = ctl->p;
    const SBank<Mixed> A = v.S[s];
    const SBank<Mixed> B = v.S[s ^ 1];
    const PBank<Mixed> P = v.P[p];
    const int ntiles = (v.n + kBlock - 1) / kBlock;
    const int tid = threadIdx.x;
    bool refresh = false;
    unsigned err = 0u;
    if (tid == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    int t = blockIdx.x;
    if (tid == 0 && t < ntiles) issue_tile(v, A, P, t, &stage[0], &full[0]);
    bool timed_out = false;
    int t_it = 0;
    for (int it = 0; t < ntiles; it++, t += gridDim.x) {
        t_it = it;
        const int b = it & 1;
        const int tn = t + gridDim.x;
        if (tid == 0 && tn < ntiles) {
            // the other buffer was released by the barrier that ended the
            // previous iteration; order those generic reads before the copy
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue_tile(v, A, P, tn, &stage[b ^ 1], &full[b ^ 1]);
        }
        const bool ok = mbar_wait_bounded(&full[b], (unsigned)(it >> 1) & 1u);
        if (__syncthreads_or(!ok)) {
            timed_out = true;
            break;
        }
        const int i = t * kBlock + tid;
        if (i < v.n) {
            const Stage& S = stage[b];
            Own o;
            o.wi = S.rot[tid];
            o.hi = S.posh[tid];
            o.li = S.posl[tid];
            o.vi = S.vel[tid];
            o.vl = S.vell[tid];
            o.wl = S.rotl[tid];
            o.rh = S.refh[tid];
            o.nn = S.nnei[tid];
            o.nw = S.nneiw[tid];
            o.nc = S.nc[tid];
            o.ncw = S.ncw[tid];
            step_one<MODEL, WCAP>(v, A, B, P, i, o, refresh, err);
        }
        __syncthreads();
    }
    if (timed_out) {
        err |= 0x80u;
        // let the copies still in flight (this iteration's tile and the next
        // one's) land before the CTA's shared memory goes away
        if (tid == 0) {
            mbar_wait_bounded(&full[t_it & 1], (unsigned)(t_it >> 1) & 1u);
            if (t + (int)gridDim.x < ntiles) mbar_wait_bounded(&full[(t_it + 1) & 1], (unsigned)((t_it + 1) >> 1) & 1u);
        }
        __syncthreads();
    }
    step_epilogue(ctl, s, refresh, err, cond, use_cond);
}

// ---------------------------------------------------------------- warp-staged
// Persistent variant with one pipeline per warp: a warp walks sub-tiles of 32
// consecutive particles, and its lane 0 brings the next sub-tile's arrays and
// its first kNeiStageRows Verlet rows into the warp's other buffer with bulk
// copies while the warp works on the current one.  Warps never wait for each
// other.  Every mbarrier wait gives up after kSpinLimit tries and sets
// GDEM_EW_TIMEOUT.
constexpr int kNeiStageRows = 8;

struct __align__(16) WStage {
    float4 posh[32], posl[32], vel[32], rot[32], vell[32], rotl[32], refh[32];
    int nnei[32], nneiw[32], nc[32], ncw[32];
    int nei[kNeiStageRows][32];
};
constexpr int kWarps = kBlock / 32;
constexpr int kWStageBytes = (int)sizeof(WStage);
static_assert(kWStageBytes % 16 == 0, "stage buffers must keep 16-byte alignment");

// Bulk copies of sub-tile `t` into `st` (lane 0).  Int arrays of the tail are
// copied in whole 16-byte units, inside their 256-byte allocation units.  The
// Verlet rows are staged only when every row k*n + 32t starts 16-byte aligned
// (n a multiple of 4); the caller reads them from HBM otherwise.
__device__ __forceinline__ void issue_sub(const View<Mixed>& v, const SBank<Mixed>& A, const PBank<Mixed>& P,
                                          int t, WStage* st, unsigned long long* bar, int nei_rows) {
    const int base = t * 32;
    const int cnt = min(32, v.n - base);
    const unsigned b16 = 16u * (unsigned)cnt;
    const unsigned b4 = 4u * (unsigned)((cnt + 3) & ~3);
    mbar_expect_tx(bar, 7u * b16 + (4u + (unsigned)nei_rows) * b4);
    bulk_g2s(st->posh, A.posh + base, b16, bar);
    bulk_g2s(st->posl, A.posl + base, b16, bar);
    bulk_g2s(st->vel, A.vel + base, b16, bar);
    bulk_g2s(st->rot, A.rot + base, b16, bar);
    bulk_g2s(st->vell, A.vell + base, b16, bar);
    bulk_g2s(st->rotl, A.rotl + base, b16, bar);
    bulk_g2s(st->refh, v.refh + base, b16, bar);
    bulk_g2s(st->nnei, v.nnei + base, b4, bar);
    bulk_g2s(st->nneiw, v.nneiw + base, b4, bar);
    bulk_g2s(st->nc, P.nc + base, b4, bar);
    bulk_g2s(st->ncw, P.ncw + base, b4, bar);
    for (int k = 0; k < nei_rows; k++) bulk_g2s(st->nei[k], v.nei + (size_t)k * v.n + base, b4, bar);
}

template <int MODEL, int WCAP>
__global__ void __launch_bounds__(kBlock, 2) k_step_mixed_wtma(View<Mixed> v, cudaGraphConditionalHandle cond,
                                                              int use_cond) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    WStage* stage = reinterpret_cast<WStage*>(smem_raw) + 2 * warp;
    __shared__ __align__(8) unsigned long long full[kWarps][2];
    Ctl* ctl = v.ctl;
    const int s = ctl->s, p = ctl->p;
    const SBank<Mixed> A = v.S[s];
    const SBank<Mixed> B = v.S[s ^ 1];
    const PBank<Mixed> P = v.P[p];
    const int nsub = (v.n + 31) / 32;
    const int stride = gridDim.x * kWarps;
    const int nei_rows = (v.n % 4 == 0) ? min(kNeiStageRows, v.nei_cap) : 0;
    bool refresh = false;
    unsigned err = 0u;
    if (lane == 0) {
        mbar_init(&full[warp][0], 1);
        mbar_init(&full[warp][1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    int t = blockIdx.x * kWarps + warp;
    if (lane == 0 && t < nsub) issue_sub(v, A, P, t, &stage[0], &full[warp][0], nei_rows);
    bool timed_out = false;
    int t_it = 0;
    for (int it = 0; t < nsub; it++, t += stride) {
        t_it = it;
        const int b = it & 1;
        const int tn = t + stride;
        if (lane == 0 && tn < nsub) {
            // the other buffer was last read before the __syncwarp that ended
            // the previous iteration; order those reads before the copy
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue_sub(v, A, P, tn, &stage[b ^ 1], &full[warp][b ^ 1], nei_rows);
        }
        const bool ok = mbar_wait_bounded(&full[warp][b], (unsigned)(it >> 1) & 1u);
        if (__any_sync(0xffffffffu, !ok)) {
            timed_out = true;
            break;
        }
        const int i = t * 32 + lane;
        if (i < v.n) {
            const WStage& S = stage[b];
            Own o;
            o.wi = S.rot[lane];
            o.hi = S.posh[lane];
            o.li = S.posl[lane];
            o.vi = S.vel[lane];
            o.vl = S.vell[lane];
            o.wl = S.rotl[lane];
            o.rh = S.refh[lane];
            o.nn = S.nnei[lane];
            o.nw = S.nneiw[lane];
            o.nc = S.nc[lane];
            o.ncw = S.ncw[lane];
            step_one<MODEL, WCAP>(v, A, B, P, i, o, refresh, err, &S.nei[0][lane], nei_rows);
        }
        __syncwarp();
    }
    if (timed_out) {
        err |= 0x80u;
        // let the copies still in flight land before the shared memory goes away
        if (lane == 0) {
            mbar_wait_bounded(&full[warp][t_it & 1], (unsigned)(t_it >> 1) & 1u);
            if (t + stride < nsub) mbar_wait_bounded(&full[warp][(t_it + 1) & 1], (unsigned)((t_it + 1) >> 1) & 1u);
        }
        __syncwarp();
    }
    step_epilogue(ctl, s, refresh, err, cond, use_cond);
}

namespace {
// MINB: resident blocks per SM the register allocation of the one-pass
// kernel is sized for (2, the default: no spills; 3: more warps in flight,
// with spills).  GDEM_MIXED_MINB picks one.  GDEM_MIXED_KERNEL=cta picks the
// CTA-staged persistent kernel, =direct the one-pass kernel, instead of the
// warp-staged persistent one.
template <int MODEL, int MINB>
void* direct_kernel_minb(int wall_cap) {
    if (wall_cap <= 16) return (void*)k_step_mixed<MODEL, 16, MINB>;
    if (wall_cap <= 32) return (void*)k_step_mixed<MODEL, 32, MINB>;
    return (void*)k_step_mixed<MODEL, 64, MINB>;
}
template <int MODEL>
void* direct_kernel(int wall_cap) {
    static const int minb = [] {
        const char* e = getenv("GDEM_MIXED_MINB");
        return e ? atoi(e) : 2;
    }();
    return minb == 3 ? direct_kernel_minb<MODEL, 3>(wall_cap) : direct_kernel_minb<MODEL, 2>(wall_cap);
}
template <int MODEL>
void* tma_kernel(int wall_cap) {
    void* fn = wall_cap <= 16   ? (void*)k_step_mixed_tma<MODEL, 16>
               : wall_cap <= 32 ? (void*)k_step_mixed_tma<MODEL, 32>
                                : (void*)k_step_mixed_tma<MODEL, 64>;
    static bool configured[3] = {false, false, false};
    const int slot = wall_cap <= 16 ? 0 : (wall_cap <= 32 ? 1 : 2);
    if (!configured[slot]) {
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * kStageBytes);
        configured[slot] = true;
    }
    return fn;
}
template <int MODEL>
void* wtma_kernel(int wall_cap) {
    void* fn = wall_cap <= 16   ? (void*)k_step_mixed_wtma<MODEL, 16>
               : wall_cap <= 32 ? (void*)k_step_mixed_wtma<MODEL, 32>
                                : (void*)k_step_mixed_wtma<MODEL, 64>;
    static bool configured[3] = {false, false, false};
    const int slot = wall_cap <= 16 ? 0 : (wall_cap <= 32 ? 1 : 2);
    if (!configured[slot]) {
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * kWarps * kWStageBytes);
        configured[slot] = true;
    }
    return fn;
}
// 0: warp-staged (default), 1: CTA-staged, 2: direct
int kernel_kind() {
    static const int k = [] {
        const char* e = getenv("GDEM_MIXED_KERNEL");
        if (e && strcmp(e, "direct") == 0) return 2;
        if (e && strcmp(e, "cta") == 0) return 1;
        return 0;
    }();
    return k;
}
int sm_count() {
    static const int c = [] {
        int dev = 0, cnt = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&cnt, cudaDevAttrMultiProcessorCount, dev);
        return cnt > 0 ? cnt : 1;
    }();
    return c;
}
}  // namespace

StepLaunch step_launch(const View<Mixed>& v) {
    const int ntiles = (v.n + kBlock - 1) / kBlock;
    const int kind = kernel_kind();
    if (kind == 0) {
        void* fn = v.mat.model == 1 ? wtma_kernel<1>(v.wall_cap) : wtma_kernel<0>(v.wall_cap);
        const int nsub = (v.n + 31) / 32;
        const int need = (nsub + kWarps - 1) / kWarps;
        const int grid = need < 2 * sm_count() ? need : 2 * sm_count();
        return StepLaunch{fn, dim3(grid), dim3(kBlock), (size_t)2 * kWarps * kWStageBytes};
    }
    if (kind == 1) {
        void* fn = v.mat.model == 1 ? tma_kernel<1>(v.wall_cap) : tma_kernel<0>(v.wall_cap);
        // two resident CTAs per SM (registers), each walking its share of tiles
        const int grid = ntiles < 2 * sm_count() ? ntiles : 2 * sm_count();
        return StepLaunch{fn, dim3(grid), dim3(kBlock), (size_t)2 * kStageBytes};
    }
    void* fn = v.mat.model == 1 ? direct_kernel<1>(v.wall_cap) : direct_kernel<0>(v.wall_cap);
    return StepLaunch{fn, dim3(ntiles), dim3(kBlock), 0};
}

void launch_step(const View<Mixed>& v, cudaStream_t st, cudaGraphConditionalHandle cond, int use_cond) {
    const StepLaunch L = step_launch(v);
    View<Mixed> vv = v;
    void* args[3] = {(void*)&vv, (void*)&cond, (void*)&use_cond};
    cudaLaunchKernel(L.fn, L.grid, L.block, args, L.smem, st);
}

}  // namespace gdem
