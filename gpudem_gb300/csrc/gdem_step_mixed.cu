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
// Compiled with multiply-add contraction on, and with the hardware's
// approximate reciprocal and square root (-prec-div=false -prec-sqrt=false).
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "gdem_step.cuh"

namespace gdem {

namespace {

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

// a - b as an unevaluated pair (s, e), exactly (Knuth's TwoSum)
__device__ __forceinline__ void two_diff(float a, float b, float& s, float& e) {
    s = __fsub_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(-b, bb));
}

// Geometry of a particle pair from the float-pair positions {hi.xyz, ±r_hi}
// and {lo.xyz, r_lo}: the relative vector rounded to FP32 (dx, dy, dz), the
// contact radius Rs = r_i + r_j and num = Rs^2 - |x_i - x_j|^2 to about FP64
// accuracy.  The high-part differences and the radius sum are split exactly
// (TwoSum), the squares exactly (FMA), and the large terms cancel in
// error-free sums, so the overlap num / (Rs + |x_ij|) carries no
// cancellation error.
struct PairGeom {
    float dx, dy, dz, Rs, num;
};
// Periodic x in FP32: the period as a float pair L = Lh + Ll and its half.
struct PerX {
    int on;
    float Lh, Ll, half;
};
// PER: the kernel is compiled for a periodic x (false: every periodic branch
// folds away at compile time)
template <bool PER, class V>
__device__ __forceinline__ PerX per_of(const V& v) {
    return PER ? PerX{v.per_x, v.Lxh, v.Lxl, v.halfLxf} : PerX{0, 0.f, 0.f, 0.f};
}
// With a periodic x, the nearest image of the high-part x separation X:
// X -/+ Lh is exact (Sterbenz: |X| lies between Lh/2 and 2 Lh), and the
// period's low part joins the error term e.
__device__ __forceinline__ void image_pair(const PerX& per, float& X, float& e) {
    if (per.on) {
        if (X > per.half) {
            X = __fsub_rn(X, per.Lh);
            e = __fsub_rn(e, per.Ll);
        } else if (X < -per.half) {
            X = __fadd_rn(X, per.Lh);
            e = __fadd_rn(e, per.Ll);
        }
    }
}
__device__ __forceinline__ PairGeom pair_geometry(float4 hi, float4 li, float4 hj, float4 lj, const PerX& per) {
    PairGeom g;
    float X, Y, Z, eX, eY, eZ;
    two_diff(hi.x, hj.x, X, eX);
    two_diff(hi.y, hj.y, Y, eY);
    two_diff(hi.z, hj.z, Z, eZ);
    image_pair(per, X, eX);
    eX = __fadd_rn(eX, __fsub_rn(li.x, lj.x));
    eY = __fadd_rn(eY, __fsub_rn(li.y, lj.y));
    eZ = __fadd_rn(eZ, __fsub_rn(li.z, lj.z));
    float S, eS;
    two_diff(fabsf(hi.w), -fabsf(hj.w), S, eS);
    const float Rl = __fadd_rn(eS, __fadd_rn(li.w, lj.w));
    const float p0 = __fmul_rn(S, S), e0 = __fmaf_rn(S, S, -p0);
    const float p1 = __fmul_rn(X, X), e1 = __fmaf_rn(X, X, -p1);
    const float p2 = __fmul_rn(Y, Y), e2 = __fmaf_rn(Y, Y, -p2);
    const float p3 = __fmul_rn(Z, Z), e3 = __fmaf_rn(Z, Z, -p3);
    float a, t1, t2, t3;
    two_diff(p0, p1, a, t1);
    two_diff(a, p2, a, t2);
    two_diff(a, p3, a, t3);
    const float small = __fadd_rn(__fadd_rn(__fadd_rn(t1, t2), t3), __fsub_rn(__fsub_rn(__fsub_rn(e0, e1), e2), e3));
    const float cross = __fsub_rn(__fmul_rn(S, Rl), __fadd_rn(__fadd_rn(__fmul_rn(X, eX), __fmul_rn(Y, eY)), __fmul_rn(Z, eZ)));
    g.num = __fadd_rn(a, __fadd_rn(small, __fmul_rn(2.f, cross)));
    g.dx = __fadd_rn(X, eX);
    g.dy = __fadd_rn(Y, eY);
    g.dz = __fadd_rn(Z, eZ);
    g.Rs = __fadd_rn(S, Rl);
    return g;
}

// First contact test on the high parts alone (one gather per candidate):
// 1 surely in contact, 0 surely not, -1 undecided (within `delta`, the bound
// on what the low parts can move the distance, of touching).
__device__ __forceinline__ int contact_hint(float4 hi, float4 hj, float delta, const PerX& per) {
    if (!(hj.w > 0.f)) return 0;  // partner inactive or leaving the box
    float dx = hi.x - hj.x;
    const float dy = hi.y - hj.y, dz = hi.z - hj.z;
    if (per.on) dx = dx > per.half ? dx - per.Lh : (dx < -per.half ? dx + per.Lh : dx);
    const float Rs = hi.w + hj.w;
    const float d2 = dx * dx + dy * dy + dz * dz;
    const float Rin = Rs - delta, Rout = Rs + delta;
    if (Rin > 0.f && d2 < Rin * Rin * 0.9999981f) return 1;
    if (d2 > Rout * Rout * 1.0000019f) return 0;
    return -1;
}

// The exact contact test (pair_geometry's num > 0) for the few candidates the
// high parts leave undecided; kept out of line so the scan loop stays small.
__device__ __noinline__ bool exact_contact(float4 hi, float4 li, float4 hj, float4 lj, PerX per) {
    return pair_geometry(hi, li, hj, lj, per).num > 0.f;
}

// a + b as an unevaluated pair (s, e), exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) { two_diff(a, -b, s, e); }

// a * b as an unevaluated pair (p, e), exactly (FMA)
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
    p = __fmul_rn(a, b);
    e = __fmaf_rn(a, b, -p);
}

// Overlap (r_h + r_l) - dist of the sphere centred at ph + pl with the feature
// of triangle T that closest_feature_f picked (kind, and t on an edge), to
// about FP64 accuracy.  The centre minus the closest point is formed as float
// pairs from corner 0 and the two edges from it (high parts in T, low parts in
// L); on a face its normal component comes from error-free products with the
// unit normal as a pair, on an edge or corner its squared length from
// error-free squares, and the overlap is (r^2 - |u|^2) / (r + |u|) without
// cancellation.  An edge's distance is stationary in t, so the FP32 t costs
// nothing to first order.  Only contacts come here.
__device__ __forceinline__ float wall_overlap(float3 ph, float3 pl, float rh, float rl, const TriRecF& T,
                                           const TriLoF& L, int kind, float t) {
    const float P[3] = {ph.x, ph.y, ph.z}, Pl[3] = {pl.x, pl.y, pl.z};
    float qh[3], ql[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float e;
        two_diff(P[k], T.v0h[k], qh[k], e);
        ql[k] = __fadd_rn(e, __fsub_rn(Pl[k], T.v0l[k]));
    }
    if (kind == 0) {
        float s, lo, p, e;
        two_prod(T.n[0], qh[0], s, lo);
#pragma unroll
        for (int k = 1; k < 3; k++) {
            float pe;
            two_prod(T.n[k], qh[k], p, pe);
            two_sum(s, p, s, e);
            lo = __fadd_rn(lo, __fadd_rn(e, pe));
        }
#pragma unroll
        for (int k = 0; k < 3; k++)
            lo = __fadd_rn(lo, __fadd_rn(__fmul_rn(T.n[k], ql[k]), __fmul_rn(L.nl[k], qh[k])));
        if (s < 0.f) {
            s = -s;
            lo = -lo;
        }
        float dh, de;
        two_diff(rh, s, dh, de);
        return __fadd_rn(dh, __fadd_rn(de, __fsub_rn(rl, lo)));
    }
    float uh[3], ul[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float ah = qh[k], al = ql[k], e;
        if (kind == 2 || kind == 4) {  // from corner 1
            two_diff(ah, T.e01[k], ah, e);
            al = __fadd_rn(al, __fsub_rn(e, L.e01l[k]));
        } else if (kind == 3) {        // corner 2
            two_diff(ah, T.e02[k], ah, e);
            al = __fadd_rn(al, __fsub_rn(e, L.e02l[k]));
        }
        if (kind >= 4) {
            float eh, el;
            if (kind == 4) {
                two_diff(T.e02[k], T.e01[k], eh, e);
                el = __fadd_rn(e, __fsub_rn(L.e02l[k], L.e01l[k]));
            } else if (kind == 5) {
                eh = T.e02[k];
                el = L.e02l[k];
            } else {
                eh = T.e01[k];
                el = L.e01l[k];
            }
            float pt, et;
            two_prod(t, eh, pt, et);
            two_diff(ah, pt, ah, e);
            al = __fadd_rn(al, __fsub_rn(__fsub_rn(e, et), __fmul_rn(t, el)));
        }
        uh[k] = ah;
        ul[k] = al;
    }
    float D, lo, p, pe, e;
    two_prod(uh[0], uh[0], D, lo);
#pragma unroll
    for (int k = 1; k < 3; k++) {
        two_prod(uh[k], uh[k], p, pe);
        two_sum(D, p, D, e);
        lo = __fadd_rn(lo, __fadd_rn(e, pe));
    }
    const float cross = __fadd_rn(__fadd_rn(__fmul_rn(uh[0], ul[0]), __fmul_rn(uh[1], ul[1])), __fmul_rn(uh[2], ul[2]));
    lo = __fadd_rn(lo, __fmul_rn(2.f, cross));
    float R2, R2e, nh, ne;
    two_prod(rh, rh, R2, R2e);
    two_diff(R2, D, nh, ne);
    const float num = __fadd_rn(nh, __fadd_rn(ne, __fsub_rn(__fadd_rn(R2e, __fmul_rn(2.f, __fmul_rn(rh, rl))), lo)));
    return num / (rh + sqrtf(D));
}

}  // namespace

// Refresh votes of a thread: the list rows (bit 0) and the inner rows (bit 1).
constexpr unsigned kVoteLists = 1u, kVoteInner = 2u;

// End of a step kernel: refresh votes, error bits, and in the last CTA the
// bank flip, the step count and the graph's rebuild conditions (list rebuild;
// inner rows, when use_cond has bit 1).
__device__ __forceinline__ void step_epilogue(Ctl* ctl, int s, unsigned votes, unsigned err,
                                              cudaGraphConditionalHandle cond, cudaGraphConditionalHandle ci,
                                              int use_cond) {
    const unsigned wv = __reduce_or_sync(0xffffffffu, votes);
    if ((threadIdx.x & 31) == 0) {
        if (wv & kVoteLists) atomicOr(&ctl->refresh, 1u);
        if (wv & kVoteInner) atomicOr(&ctl->irefresh, 1u);
    }
    if (err) atomicOr(&ctl->error, err);
    if (last_block(&ctl->done[0])) {
        if (threadIdx.x == 0) {
            ctl->done[0] = 0;
            ctl->work = 0;
            ctl->s = s ^ 1;
            ctl->steps += 1ull;
            const unsigned r = atomicAdd(&ctl->refresh, 0u);
            if (use_cond) cudaGraphSetConditional(cond, r ? 1u : 0u);
            if (use_cond & 2) cudaGraphSetConditional(ci, atomicAdd(&ctl->irefresh, 0u) ? 1u : 0u);
        }
    }
}

// State of one particle at the start of a step (bank s), however it was
// brought in: straight from HBM, or staged in shared memory by bulk copies.
struct Own {
    float4 wi, hi, li, vi, vl, wl, rh;
    int nn, nw, nc, ncw;
};

// Per-particle contact constants (Hertz-Mindlin: the scene's friction and
// damping, per particle when the engine has per-particle materials).
struct Mat {
    float ki, etai, sqrtmi, invmoi;
    float mu, damp;
};

template <int MODEL>
__device__ __forceinline__ Mat own_material(const View<Mixed>& v, const PBank<Mixed>& P, int i, float ri,
                                            float invmi) {
    Mat m;
    if (MODEL == 0) {
        const float4 mi = __ldg(&P.mat[i]);
        m.ki = mi.x; m.etai = mi.y; m.sqrtmi = mi.z; m.invmoi = mi.w;
        m.mu = v.muf;
        m.damp = 0.f;
    } else {
        m.ki = m.etai = m.sqrtmi = 0.f;
        m.invmoi = 2.5f * invmi / (ri * ri);  // 1 / (2/5 m r^2)
        if (v.per_particle_mat) {
            const float4 mi = __ldg(&P.mat[i]);
            m.mu = mi.x;
            m.damp = mi.y;
        } else {
            m.mu = v.muf;
            m.damp = v.damp_cf;
        }
    }
    return m;
}

struct Force6 {
    float fx, fy, fz, mx, my, mz;
};

// Force and torque on i from one particle contact (calc_normal_force /
// calc_tangential_force, cpu_dem.cu:953, :783, or the Hertz-Mindlin law),
// with the spring history (sp, cp) of the contact updated in place.
template <int MODEL>
__device__ __forceinline__ Force6 pair_force(const View<Mixed>& v, const PairGeom& g, float ri, float rj,
                                             float4 vi, float4 wi, float4 vj, float4 wj, float invmi, const Mat& m,
                                             Vec3<float>& sp, Vec3<float>& cp) {
    using R = float;
    const R dx = g.dx, dy = g.dy, dz = g.dz;
    const R distsq = dx * dx + dy * dy + dz * dz;
    const R Rs = g.Rs;
    const R dist = sqrtf(distsq);
    const R inv = 1.f / dist;
    // the overlap Rs - dist without its cancellation: (Rs^2 - d^2) / (Rs + d)
    const R delMag = g.num / (Rs + dist);
    const R nx = dx * inv, ny = dy * inv, nz = dz * inv;
    const R vrx = vi.x - vj.x, vry = vi.y - vj.y, vrz = vi.z - vj.z;
    const R vdn = vrx * nx + vry * ny + vrz * nz;
    const R vnx = vdn * nx, vny = vdn * ny, vnz = vdn * nz;
    R fnx, fny, fnz, kt, gt, Rstar = 0.f;
    if (MODEL == 0) {
        const R meff = 1.f / (invmi + vj.w);
        const R eta = m.etai * sqrtf(meff);
        const R fel = m.ki * delMag;
        fnx = fel * nx - eta * vnx;
        fny = fel * ny - eta * vny;
        fnz = fel * nz - eta * vnz;
        kt = m.ki;
        gt = eta;
    } else {
        Rstar = ri * rj / Rs;
        const R mstar = 1.f / (invmi + vj.w);
        const R sqrtRd = sqrtf(Rstar * delMag);
        const R fel = v.kn_cf * sqrtRd * delMag;
        const R gn = m.damp * sqrtf(v.sn_cf * sqrtRd * mstar);
        const R fnm = fel - gn * vdn;
        fnx = fnm * nx;
        fny = fnm * ny;
        fnz = fnm * nz;
        kt = v.kt_cf * sqrtRd;
        gt = m.damp * sqrtf(kt * mstar);
    }
    const R ax_ = ri * wi.x + rj * wj.x;
    const R ay_ = ri * wi.y + rj * wj.y;
    const R az_ = ri * wi.z + rj * wj.z;
    const R vtx = (vrx - vnx) + (ay_ * nz - az_ * ny);
    const R vty = (vry - vny) + (az_ * nx - ax_ * nz);
    const R vtz = (vrz - vnz) + (ax_ * ny - ay_ * nx);
    Vec3<R> ft;
    const R fnsq = fnx * fnx + fny * fny + fnz * fnz;
    tangential<Mixed>(nx, ny, nz, fnsq, vtx, vty, vtz, gt, kt, m.mu, v.dtf, sp, cp, ft);
    Force6 F;
    F.fx = fnx + ft.x;
    F.fy = fny + ft.y;
    F.fz = fnz + ft.z;
    F.mx = ri * (ny * ft.z - nz * ft.y);
    F.my = ri * (nz * ft.x - nx * ft.z);
    F.mz = ri * (nx * ft.y - ny * ft.x);
    if (MODEL == 1 && v.mu_rollf > 0.f) {
        const R rx = wi.x - wj.x, ry = wi.y - wj.y, rz = wi.z - wj.z;
        const R wn2 = rx * rx + ry * ry + rz * rz;
        if (wn2 > 0.f) {
            const R tr = -v.mu_rollf * Rstar * sqrtf(fnsq) * rsqrtf(wn2);
            F.mx += tr * rx;
            F.my += tr * ry;
            F.mz += tr * rz;
        }
    }
    return F;
}

// Sphere centre (ph + pl) moved to its x image nearest a triangle whose first
// corner has high-part x x0h (periodic x; triangles are narrower than a
// quarter period): the shift by -/+ L is formed as a float pair.
__device__ __forceinline__ void wall_image(const PerX& per, float x0h, float3& ph, float3& pl) {
    if (!per.on) return;
    const float d = ph.x - x0h;
    if (d > per.half || d < -per.half) {
        const float sh = d > 0.f ? per.Lh : -per.Lh, sl = d > 0.f ? per.Ll : -per.Ll;
        float s, e;
        two_diff(ph.x, sh, s, e);
        ph.x = s;
        pl.x = __fadd_rn(__fsub_rn(pl.x, sl), e);
    }
}

// Force of one wall contact on particle i (after the feature dedupe), added
// to F: the normal force, then the history slot of triangle t, the
// tangential spring, its torque and the rolling resistance
// (wall_collision_verlet, cpu_dem.cu:238).
template <int MODEL>
__device__ __forceinline__ void wall_contact_force(const View<Mixed>& v, const PBank<Mixed>& P, int i, int t,
                                                   float nx, float ny, float nz, float delmag, float ri, float4 vi,
                                                   float4 wi, float invmi, const Mat& mt, int& ncw,
                                                   unsigned long long& wtouched, Force6& F, unsigned& err) {
    using T = Mixed;
    using R = float;
    const int n = v.n;
    const R vdn = vi.x * nx + vi.y * ny + vi.z * nz;
    const R vnx = vdn * nx, vny = vdn * ny, vnz = vdn * nz;
    R fnx, fny, fnz, kt, gt;
    if (MODEL == 0) {
        const R eta = mt.etai * mt.sqrtmi;
        const R fel = mt.ki * delmag;
        fnx = fel * nx - eta * vnx;
        fny = fel * ny - eta * vny;
        fnz = fel * nz - eta * vnz;
        kt = mt.ki;
        gt = eta;
    } else {
        const R mstar = 1.f / invmi;
        const R sqrtRd = sqrtf(ri * delmag);
        const R fel = v.kn_cf * sqrtRd * delmag;
        const R gn = mt.damp * sqrtf(v.sn_cf * sqrtRd * mstar);
        const R fnm = fel - gn * vdn;
        fnx = fnm * nx;
        fny = fnm * ny;
        fnz = fnm * nz;
        kt = v.kt_cf * sqrtRd;
        gt = mt.damp * sqrtf(kt * mstar);
    }
    const R ax_ = ri * wi.x, ay_ = ri * wi.y, az_ = ri * wi.z;
    const R vtx = (vi.x - vnx) + (ay_ * nz - az_ * ny);
    const R vty = (vi.y - vny) + (az_ * nx - ax_ * nz);
    const R vtz = (vi.z - vnz) + (ax_ * ny - ay_ * nx);
    F.fx += fnx;
    F.fy += fny;
    F.fz += fnz;
    bool fresh;
    const int slot = find_slot<T>(P.hwid, n, i, ncw, t, v.histw_cap, fresh);
    if (slot < 0) {
        err |= 0x8u;
        return;
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
    tangential<T>(nx, ny, nz, fnsq, vtx, vty, vtz, gt, kt, mt.mu, v.dtf, sp, cp, ft);
    F.fx += ft.x;
    F.fy += ft.y;
    F.fz += ft.z;
    F.mx += ri * (ny * ft.z - nz * ft.y);
    F.my += ri * (nz * ft.x - nx * ft.z);
    F.mz += ri * (nx * ft.y - ny * ft.x);
    if (MODEL == 1 && v.mu_rollf > 0.f) {
        const R wn2 = wi.x * wi.x + wi.y * wi.y + wi.z * wi.z;
        if (wn2 > 0.f) {
            const R tr = -v.mu_rollf * ri * sqrtf(fnsq) * rsqrtf(wn2);
            F.mx += tr * wi.x;
            F.my += tr * wi.y;
            F.mz += tr * wi.z;
        }
    }
    P.hwx[h] = sp.x; P.hwy[h] = sp.y; P.hwz[h] = sp.z;
    P.cwx[h] = cp.x; P.cwy[h] = cp.y; P.cwz[h] = cp.z;
}

// A contact's feature against the features this particle already touched
// this step: an edge or corner shared by two triangles counts once
// (wall_collision_verlet's vertex/edge list).  Face contacts (hit -1) always
// count.
template <int WCAP>
__device__ __forceinline__ bool feature_is_new(int hit, int* vore, int& nvore) {
    if (hit == -1) return true;
    for (int q = 0; q < nvore; q++)
        if (vore[q] == hit) return false;
    if (nvore < WCAP) vore[nvore++] = hit;
    return true;
}

// Wall contacts of particle i from its wall list, in list order
// (wall_collision_verlet, cpu_dem.cu:238), added to f and m.
template <int MODEL, int WCAP, bool PER>
__device__ __forceinline__ void wall_forces(const View<Mixed>& v, const PBank<Mixed>& P, int i, int nw, int ncw,
                                            float4 hi, float4 li, float4 vi, float4 wi, float invmi, const Mat& mt,
                                            Force6& F, unsigned& err) {
    using R = float;
    const int n = v.n;
    const int* __restrict__ neiw = v.neiw;
    const R ri = hi.w;
    unsigned long long wtouched = 0ull;
    int vore[WCAP];
    int nvore = 0;
    const float3 ph = make_float3(hi.x, hi.y, hi.z), pl = make_float3(li.x, li.y, li.z);
    const PerX per = per_of<PER>(v);
    // candidates within the FP32 error bound of touching go to the exact overlap
    const R rm = ri + v.wall_delta;
    const R rmsq = rm * rm;
    for (int k0 = 0; k0 < nw; k0 += 4) {
        // four candidates at a time: their indices, then the first 48 bytes
        // of their records (corner pair and normal), all in flight together,
        // for the plane-distance test that rejects most of them
        int tt[4];
#pragma unroll
        for (int q = 0; q < 4; q++) tt[q] = k0 + q < nw ? __ldg(&neiw[(size_t)(k0 + q) * n + i]) : -1;
        unsigned near = 0u;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if (tt[q] < 0) continue;
            const float4* rec = reinterpret_cast<const float4*>(&v.trif[tt[q]]);
            const float4 a = __ldg(rec), b = __ldg(rec + 1), c = __ldg(rec + 2);
            // a = {v0h.xyz, v0l.x}, b = {v0l.yz, n.xy}, c = {n.z, ...}
            float3 qh = ph, ql = pl;
            wall_image(per, a.x, qh, ql);
            const float ax = (qh.x - a.x) + (ql.x - a.w);
            const float ay = (ph.y - a.y) + (pl.y - b.x);
            const float az = (ph.z - a.z) + (pl.z - b.y);
            const float dist = b.z * ax + b.w * ay + c.x * az;
            if (!(dist * dist > rmsq)) near |= 1u << q;
        }
        while (near) {
            const int q = __ffs(near) - 1;
            near &= near - 1u;
            const int t = __ldg(&neiw[(size_t)(k0 + q) * n + i]);
            float3 qh = ph, ql = pl;
            wall_image(per, v.trif[t].v0h[0], qh, ql);
            const FeatureF f = closest_feature_f(qh, ql, rmsq, v.trif[t]);
            if (!(f.dist < rm)) continue;
            const R delmag = wall_overlap(qh, ql, ri, li.w, v.trif[t], v.trilo[t], f.kind, f.t);
            if (!(delmag > 0.f)) continue;
            if (!feature_is_new<WCAP>(f.hit, vore, nvore)) continue;
            wall_contact_force<MODEL>(v, P, i, t, f.nx, f.ny, f.nz, delmag, ri, vi, wi, invmi, mt, ncw, wtouched, F,
                                      err);
        }
    }
    P.ncw[i] = surviving(wtouched, ncw);
}

// Inactive particle, or one that left the box last step (status 2): frozen
// from now on.
__device__ __forceinline__ void freeze_one(const View<Mixed>& v, const SBank<Mixed>& B, int i, const Own& o) {
    float4 hi = o.hi, wi = o.wi;
    hi.w = -fabsf(hi.w);
    B.posh[i] = hi;
    B.posl[i] = o.li;
    B.vel[i] = o.vi;
    B.vell[i] = o.vl;
    B.rotl[i] = o.wl;
    wi.w = 0.f;
    B.rot[i] = wi;
    if (v.store_forces) {
        v.fx[i] = 0.; v.fy[i] = 0.; v.fz[i] = 0.;
        v.tx[i] = 0.; v.ty[i] = 0.; v.tz[i] = 0.;
    }
}

// Symplectic Euler (cpu_dem.cu:1622-1652) on the float pairs of position,
// velocity and spin, so their many small increments do not round away; the
// refresh and out-of-box tests; the new state into bank s^1.
template <bool PER>
__device__ __forceinline__ void integrate_one(const View<Mixed>& v, const SBank<Mixed>& B, int i, const Own& o,
                                              float invmoi, const Force6& F, unsigned& votes, unsigned& err) {
    using R = float;
    const PerX per = per_of<PER>(v);
    const R dt = v.dtf;
    const R invmi = o.vi.w;
    float4 vl = o.vl, wl = o.wl;
    float nvx = o.vi.x, nvy = o.vi.y, nvz = o.vi.z;
    pair_add(nvx, vl.x, (F.fx * invmi + v.gxf) * dt);
    pair_add(nvy, vl.y, (F.fy * invmi + v.gyf) * dt);
    pair_add(nvz, vl.z, (F.fz * invmi + v.gzf) * dt);
    // displacement v*dt as a float pair (the product's rounding error by FMA)
    const R sx = nvx * dt, sy = nvy * dt, sz = nvz * dt;
    const R ex_ = fmaf(nvx, dt, -sx) + vl.x * dt;
    const R ey_ = fmaf(nvy, dt, -sy) + vl.y * dt;
    const R ez_ = fmaf(nvz, dt, -sz) + vl.z * dt;
    float4 nh = o.hi, nl = o.li;
    pair_add(nh.x, nl.x, sx);
    pair_add(nh.y, nl.y, sy);
    pair_add(nh.z, nl.z, sz);
    nl.x += ex_;
    nl.y += ey_;
    nl.z += ez_;
    // periodic x: back into the period.  Only a centre within two ulps of a
    // face can have crossed it; those take the exact FP64 test and shift.
    if (per.on && (nh.x > v.perf[1] || nh.x < v.perf[0])) {
        double x = (double)nh.x + (double)nl.x;
        if (x >= v.maxx) x -= v.Lx;
        else if (x < v.minx) x += v.Lx;
        nh.x = __double2float_rn(x);
        nl.x = __double2float_rn(x - (double)nh.x);
    }
    float nwx = o.wi.x, nwy = o.wi.y, nwz = o.wi.z;
    pair_add(nwx, wl.x, F.mx * invmoi * dt);
    pair_add(nwy, wl.y, F.my * invmoi * dt);
    pair_add(nwz, wl.z, F.mz * invmoi * dt);
    B.vell[i] = vl;
    B.rotl[i] = wl;
    // refresh tests against the positions of the last list rebuild and of the
    // last inner rows, on the high parts: they only decide when rows are
    // rebuilt, and each threshold leaves a margin of half its skin to its
    // cutoff.  The votes are sticky: the persistent kernels integrate many
    // particles per thread.
    {
        R ex = nh.x - o.rh.x;
        if (per.on) ex = ex > per.half ? ex - per.Lh : (ex < -per.half ? ex + per.Lh : ex);
        const R ey = nh.y - o.rh.y, ez = nh.z - o.rh.z;
        if (ex * ex + ey * ey + ez * ez > v.thresh_sqf) votes |= kVoteLists;
    }
    if (v.inner_on) {
        const float4 rf = v.refi[i];
        R ex = nh.x - rf.x;
        if (per.on) ex = ex > per.half ? ex - per.Lh : (ex < -per.half ? ex + per.Lh : ex);
        const R ey = nh.y - rf.y, ez = nh.z - rf.z;
        if (ex * ex + ey * ey + ez * ez > v.inner_thresh_sqf) votes |= kVoteInner;
    }
    // out of bounds (the box rounded outwards to FP32; not in a periodic x)
    R status = 1.f;
    if ((!per.on && (nh.x < v.boxf[0] || nh.x > v.boxf[3])) || nh.y < v.boxf[1] || nh.y > v.boxf[4] ||
        nh.z < v.boxf[2] || nh.z > v.boxf[5])
        status = 2.f;
    if (!(nvx == nvx && nvy == nvy && nvz == nvz)) {
        err |= 0x20u;
        status = 2.f;
    }
    nh.w = status == 1.f ? fabsf(o.hi.w) : -fabsf(o.hi.w);
    B.posh[i] = nh;
    B.posl[i] = nl;
    B.vel[i] = make_float4(nvx, nvy, nvz, invmi);
    B.rot[i] = make_float4(nwx, nwy, nwz, status);
    if (v.store_forces) {
        v.fx[i] = F.fx; v.fy[i] = F.fy; v.fz[i] = F.fz;
        v.tx[i] = F.mx; v.ty[i] = F.my; v.tz[i] = F.mz;
    }
}

// One particle's step, one thread: particle contacts in row order (the row
// read four entries at a time so their gathers are in flight together), wall
// contacts, integration.  Writes bank s^1 and the history.
template <int MODEL, int WCAP, bool PER>
__device__ __forceinline__ void step_one(const View<Mixed>& v, const SBank<Mixed>& A, const SBank<Mixed>& B,
                                         const PBank<Mixed>& P, int i, const Own& o, unsigned& votes, unsigned& err,
                                         const int* nei_s = nullptr, int nei_s_rows = 0) {
    using T = Mixed;
    using R = float;
    if (o.wi.w != 1.f) {
        freeze_one(v, B, i, o);
        return;
    }
    const int n = v.n;
    const PerX per = per_of<PER>(v);
    const float4* __restrict__ Aposh = A.posh;
    const float4* __restrict__ Aposl = A.posl;
    const float4* __restrict__ Avel = A.vel;
    const float4* __restrict__ Arot = A.rot;
    const int* __restrict__ nei = v.nei;
    const float4 hi = o.hi, li = o.li;
    const R ri = hi.w;
    const R invmi = o.vi.w;
    const Mat mt = own_material<MODEL>(v, P, i, ri, invmi);
    Force6 F = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int nc = o.nc;
    const int nn = o.nn;
    unsigned long long touched = 0ull;
    for (int k0 = 0; k0 < nn; k0 += 4) {
        int jj[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int k = k0 + q;
            jj[q] = k < nn ? (int)((unsigned)(k < nei_s_rows ? nei_s[k * 32] : __ldg(&nei[(size_t)k * n + i])) & v.row_mask)
                           : -1;
        }
        float4 hj[4];
#pragma unroll
        for (int q = 0; q < 4; q++)
            if (jj[q] >= 0) hj[q] = __ldg(&Aposh[jj[q]]);
        unsigned hit = 0u;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if (jj[q] < 0) continue;
            const int h = contact_hint(hi, hj[q], v.nb_delta, per);
            if (h > 0 || (h < 0 && exact_contact(hi, li, hj[q], __ldg(&Aposl[jj[q]]), per))) hit |= 1u << q;
        }
        while (hit) {
            const int q = __ffs(hit) - 1;
            hit &= hit - 1u;
            const int k = k0 + q;
            const int j = (int)((unsigned)(k < nei_s_rows ? nei_s[k * 32] : __ldg(&nei[(size_t)k * n + i])) & v.row_mask);
            const float4 hjq = __ldg(&Aposh[j]), ljq = __ldg(&Aposl[j]);
            bool fresh;
            const int slot = find_slot<T>(P.hid, n, i, nc, j, v.hist_cap, fresh);
            if (slot < 0) {
                err |= 0x4u;
                continue;
            }
            const size_t h = (size_t)slot * n + i;
            Vec3<R> sp, cp;
            if (fresh) {
                P.hid[h] = j;
                sp.x = sp.y = sp.z = 0.f;
                cp.x = cp.y = cp.z = 0.f;
            } else {
                sp.x = P.hx[h]; sp.y = P.hy[h]; sp.z = P.hz[h];
                cp.x = P.cx[h]; cp.y = P.cy[h]; cp.z = P.cz[h];
            }
            touched |= 1ull << slot;
            const Force6 G = pair_force<MODEL>(v, pair_geometry(hi, li, hjq, ljq, per), ri, hjq.w, o.vi, o.wi, __ldg(&Avel[j]), __ldg(&Arot[j]),
                                               invmi, mt, sp, cp);
            F.fx += G.fx; F.fy += G.fy; F.fz += G.fz;
            F.mx += G.mx; F.my += G.my; F.mz += G.mz;
            P.hx[h] = sp.x; P.hy[h] = sp.y; P.hz[h] = sp.z;
            P.cx[h] = cp.x; P.cy[h] = cp.y; P.cz[h] = cp.z;
        }
    }
    P.nc[i] = surviving(touched, nc);
    wall_forces<MODEL, WCAP, PER>(v, P, i, o.nw, o.ncw, hi, li, o.vi, o.wi, invmi, mt, F, err);
    integrate_one<PER>(v, B, i, o, mt.invmoi, F, votes, err);
}

// One thread per particle, state loaded straight from HBM.
template <int MODEL, int WCAP, int MINB, bool PER>
__global__ void __launch_bounds__(kBlock, MINB) k_step_mixed(View<Mixed> v, cudaGraphConditionalHandle cond, cudaGraphConditionalHandle cond_inner,
                                                            int use_cond) {
    Ctl* ctl = v.ctl;
    const int s = ctl->s, p = ctl->p;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const SBank<Mixed> A = v.S[s];
    const SBank<Mixed> B = v.S[s ^ 1];
    const PBank<Mixed> P = v.P[p];
    unsigned votes = 0u;
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
        step_one<MODEL, WCAP, PER>(v, A, B, P, i, o, votes, err);
    }
    step_epilogue(ctl, s, votes, err, cond, cond_inner, use_cond);
}

// ---------------------------------------------------------------- bulk copies
// Bulk copies (cp.async.bulk) into shared memory with completion counted on
// an mbarrier.  Every wait on an mbarrier gives up after kSpinLimit tries
// (View::wait_tries for the pipeline waits) and the kernel then sets
// GDEM_EW_TIMEOUT.  After a pipeline wait gave up, the waits for the copies
// still in flight keep the full kSpinLimit, so no CTA leaves a copy
// outstanding when its shared memory goes away.

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
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  unsigned tries = kSpinLimit) {
    for (unsigned k = 0; k < tries; k++)
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
// ---------------------------------------------------------------- warp-staged
// Persistent variant with one pipeline per warp: a warp walks sub-tiles of 32
// consecutive particles, and its lane 0 brings the next sub-tile's arrays and
// its first kNeiStageRows Verlet rows into the warp's other buffer with bulk
// copies while the warp works on the current one.  Warps never wait for each
// other.  Every mbarrier wait gives up after kSpinLimit tries and sets
// GDEM_EW_TIMEOUT.
constexpr int kNeiStageRows = 1;

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

template <int MODEL, int WCAP, bool PER>
__global__ void __launch_bounds__(kBlock, 2) k_step_mixed_wtma(View<Mixed> v, cudaGraphConditionalHandle cond, cudaGraphConditionalHandle cond_inner,
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
    unsigned votes = 0u;
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
        const bool ok = mbar_wait_bounded(&full[warp][b], (unsigned)(it >> 1) & 1u, v.wait_tries);
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
            step_one<MODEL, WCAP, PER>(v, A, B, P, i, o, votes, err, &S.nei[0][lane], nei_rows);
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
    step_epilogue(ctl, s, votes, err, cond, cond_inner, use_cond);
}

// ---------------------------------------------------------------- warp-cooperative
// The warp-staged pipeline with the particle contacts computed by the whole
// warp.  Every lane first tests its whole Verlet row (a bit per entry in
// contact).  Then, kCoopQ contacts per lane at a time, it finds their history
// slots in row order (the entry's slot hint checked against the key, else a
// search) and queues them; the warp computes the queued contacts 32 at a
// time, whoever owns them, and each lane adds its own contacts' results back
// in row order.  The contact law runs with every lane busy, and its gathers
// and history loads are in flight together instead of one contact after
// another.  Shared memory per warp is kept small (two stage buffers and the
// queue, 6.9 KB) so that five CTAs of four warps share an SM with a large
// L1 beside them for the neighbour and history gathers: staging the first
// history-key rows in shared memory as well measured slower (0.463 ms on the
// 1M bed with three rows, 0.496 with seven, against 0.452 with none).
constexpr int kCoopWarps = 4;
constexpr int kCoopQ = 2;

struct __align__(16) CStage {
    float4 posh[32], posl[32], vel[32], rot[32];
    int nnei[32], nneiw[32], nc[32], ncw[32];
    int nei[kNeiStageRows][32];
};
static_assert(sizeof(CStage) % 16 == 0, "stage buffers must keep 16-byte alignment");

// The warp's contact queue: a ring the lanes fill kCoopQ contacts each per
// round and the warp drains 32 at a time (positions grow without bound; the
// slot of position x is x % kRing).  The queue holds fewer than 32 before a
// round adds at most 64, so kRing = 96 never overflows.
constexpr int kRing = 3 * 32;
struct __align__(16) CQueue {
    int j[kRing];             // partner's storage index
    int pk[kRing];            // history slot | fresh << 6 | owning lane << 7
    float f[6][32];           // force and torque of each contact of the batch being drained
    unsigned owned[32];       // the positions of a drained batch each lane owns (bit b: head + b)
};

constexpr size_t kCoopSmem = 2 * kCoopWarps * sizeof(CStage) + kCoopWarps * sizeof(CQueue);

__device__ __forceinline__ void bulk_prefetch_l2(const void* src, unsigned bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// Bulk copies of sub-tile `t` into `st` (lane 0): positions, velocities,
// spins and counts, plus the first Verlet rows when every row k*n + 32t
// starts 16-byte aligned (n a multiple of 4).  The
// arrays read only at the end of the sub-tile (low parts, reference
// positions of the list and inner rows) are prefetched into L2.
__device__ __forceinline__ void issue_csub(const View<Mixed>& v, const SBank<Mixed>& A, const PBank<Mixed>& P,
                                           int t, CStage* st, unsigned long long* bar, int nei_rows) {
    const int base = t * 32;
    const int cnt = min(32, v.n - base);
    const unsigned b16 = 16u * (unsigned)cnt;
    const unsigned b4 = 4u * (unsigned)((cnt + 3) & ~3);
    mbar_expect_tx(bar, 4u * b16 + (4u + (unsigned)nei_rows) * b4);
    bulk_g2s(st->posh, A.posh + base, b16, bar);
    bulk_g2s(st->posl, A.posl + base, b16, bar);
    bulk_g2s(st->vel, A.vel + base, b16, bar);
    bulk_g2s(st->rot, A.rot + base, b16, bar);
    bulk_g2s(st->nnei, v.nnei + base, b4, bar);
    bulk_g2s(st->nneiw, v.nneiw + base, b4, bar);
    bulk_g2s(st->nc, P.nc + base, b4, bar);
    bulk_g2s(st->ncw, P.ncw + base, b4, bar);
    for (int k = 0; k < nei_rows; k++) bulk_g2s(st->nei[k], v.nei + (size_t)k * v.n + base, b4, bar);
    bulk_prefetch_l2(A.vell + base, b16);
    bulk_prefetch_l2(A.rotl + base, b16);
    bulk_prefetch_l2(v.refh + base, b16);
    if (v.inner_on) bulk_prefetch_l2(v.refi + base, b16);
}

// The wall contacts of a warp's sub-tile with the geometry spread over the
// warp: the lanes' wall rows, one after another, are taken 32 candidates at
// a time, one per lane, through the closest feature and the exact overlap
// (their record loads in flight together instead of one candidate after
// another on the few lanes that have any); each lane then takes its own
// candidates in row order through the feature dedupe and the force, so its
// sums are those of wall_forces.  The batch results pass through the
// queue's result buffer.  A lane's own state and material are read only
// where it has a contact, so none of it is held in registers across the
// geometry (which removed the kernel's register spills).  All lanes call it;
// nw is 0 on inactive lanes.
template <int MODEL, int WCAP, bool PER>
__device__ __forceinline__ void coop_walls(const View<Mixed>& v, const PBank<Mixed>& P, const CStage& S, CQueue* que,
                                           int t, int lane, bool active, int nw, int ncw, Force6& F, unsigned& err) {
    const int n = v.n;
    const PerX per = per_of<PER>(v);
    int incl = nw;
#pragma unroll
    for (int o2 = 1; o2 < 32; o2 <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o2);
        if (lane >= o2) incl += y;
    }
    const int excl = incl - nw;
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int i = t * 32 + lane;
    unsigned long long wtouched = 0ull;
    int vore[WCAP];
    int nvore = 0;
    for (int base = 0; base < total; base += 32) {
        const int c = base + lane;
        // the candidate's owner: the first lane whose running count passes c
        int ow = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1)
            if (__shfl_sync(0xffffffffu, incl, ow + step - 1) <= c) ow += step;
        const int k = c - __shfl_sync(0xffffffffu, excl, ow);
        int hit = -3, tri = 0;
        float nx = 0.f, ny = 0.f, nz = 0.f, dm = 0.f;
        if (c < total) {
            tri = __ldg(&v.neiw[(size_t)k * n + t * 32 + ow]);
            const float4 hiw = S.posh[ow], liw = S.posl[ow];
            const float rm = hiw.w + v.wall_delta;
            float3 qh = make_float3(hiw.x, hiw.y, hiw.z), ql = make_float3(liw.x, liw.y, liw.z);
            wall_image(per, v.trif[tri].v0h[0], qh, ql);
            // beyond rm the plane test inside rejects it, as the prefilter of
            // wall_forces does
            const FeatureF f = closest_feature_f(qh, ql, rm * rm, v.trif[tri]);
            if (f.dist < rm) {
                const float d = wall_overlap(qh, ql, hiw.w, liw.w, v.trif[tri], v.trilo[tri], f.kind, f.t);
                if (d > 0.f) {
                    hit = f.hit;
                    nx = f.nx;
                    ny = f.ny;
                    nz = f.nz;
                    dm = d;
                }
            }
        }
        que->f[0][lane] = nx;
        que->f[1][lane] = ny;
        que->f[2][lane] = nz;
        que->f[3][lane] = dm;
        que->f[4][lane] = __int_as_float(hit);
        que->f[5][lane] = __int_as_float(tri);
        __syncwarp();
        // this lane's candidates in the batch, in row order
        const int y1 = min(incl, base + 32) - base;
        for (int y = max(excl, base) - base; y < y1; y++) {
            const int fh = __float_as_int(que->f[4][y]);
            if (fh == -3) continue;
            if (!feature_is_new<WCAP>(fh, vore, nvore)) continue;
            // this lane's state and material, read only where it has a contact
            const float4 hi = S.posh[lane], vi = S.vel[lane], wi = S.rot[lane];
            const Mat mt = own_material<MODEL>(v, P, i, hi.w, vi.w);
            wall_contact_force<MODEL>(v, P, i, __float_as_int(que->f[5][y]), que->f[0][y], que->f[1][y],
                                      que->f[2][y], que->f[3][y], hi.w, vi, wi, vi.w, mt, ncw, wtouched, F, err);
        }
        __syncwarp();
    }
    if (active) P.ncw[i] = surviving(wtouched, ncw);
}

template <int MODEL, int WCAP, int MINB, bool PER>
__global__ void __launch_bounds__(kCoopWarps * 32, MINB) k_step_mixed_coop(View<Mixed> v, cudaGraphConditionalHandle cond, cudaGraphConditionalHandle cond_inner,
                                                                    int use_cond) {
    using R = float;
    constexpr int Q = kCoopQ;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    CStage* stage = reinterpret_cast<CStage*>(smem_raw) + 2 * warp;
    CQueue* que = reinterpret_cast<CQueue*>(smem_raw + 2 * kCoopWarps * sizeof(CStage)) + warp;
    __shared__ __align__(8) unsigned long long full[kCoopWarps][2];
    Ctl* ctl = v.ctl;
    const int s = ctl->s, p = ctl->p;
    const SBank<Mixed> A = v.S[s];
    const SBank<Mixed> B = v.S[s ^ 1];
    const PBank<Mixed> P = v.P[p];
    const float4* __restrict__ Aposh = A.posh;
    const float4* __restrict__ Aposl = A.posl;
    const float4* __restrict__ Avel = A.vel;
    const float4* __restrict__ Arot = A.rot;
    const int* __restrict__ nei = v.nei;
    const int n = v.n;
    const int nsub = (n + 31) / 32;
    const int nei_rows = (n % 4 == 0) ? min(kNeiStageRows, v.nei_cap) : 0;
    const unsigned rmask = v.row_mask;
    const PerX per = per_of<PER>(v);
    unsigned votes = 0u;
    unsigned err = 0u;
    if (lane == 0) {
        mbar_init(&full[warp][0], 1);
        mbar_init(&full[warp][1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    // sub-tiles are handed out one at a time from a counter, so warps that
    // meet dense sub-tiles (many contacts, many wall candidates) take fewer
    int t = 0;
    if (lane == 0) {
        t = (int)atomicAdd(&ctl->work, 1u);
        if (t < nsub) issue_csub(v, A, P, t, &stage[0], &full[warp][0], nei_rows);
    }
    t = __shfl_sync(0xffffffffu, t, 0);
    bool timed_out = false;
    int t_it = 0, t_next = nsub;
    for (int it = 0; t < nsub; it++, t = t_next) {
        t_it = it;
        const int b = it & 1;
        int tn = 0;
        if (lane == 0) tn = (int)atomicAdd(&ctl->work, 1u);
        tn = __shfl_sync(0xffffffffu, tn, 0);
        t_next = tn;
        if (lane == 0 && tn < nsub) {
            // the other buffer was last read before the __syncwarp that ended
            // the previous iteration; order those reads before the copy
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue_csub(v, A, P, tn, &stage[b ^ 1], &full[warp][b ^ 1], nei_rows);
        }
        const bool ok = mbar_wait_bounded(&full[warp][b], (unsigned)(it >> 1) & 1u, v.wait_tries);
        if (__any_sync(0xffffffffu, !ok)) {
            timed_out = true;
            break;
        }
        CStage& S = stage[b];
        const int i = t * 32 + lane;
        const bool valid = i < n;
        const bool active = valid && S.rot[lane].w == 1.f;
        if (valid && !active) {
            Own o;
            o.wi = S.rot[lane];
            o.hi = S.posh[lane];
            o.li = S.posl[lane];
            o.vi = S.vel[lane];
            o.vl = __ldg(&A.vell[i]);
            o.wl = __ldg(&A.rotl[i]);
            freeze_one(v, B, i, o);
        }
        Force6 F = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        int nc = S.nc[lane];
        unsigned long long touched = 0ull;
        const int nn = active ? S.nnei[lane] : 0;
        const int* nei_s = &S.nei[0][lane];
        // ---- this lane's whole row in one pass, four entries at a time with
        // their gathers in flight together: a bit per row entry in contact
        unsigned long long hit_lo = 0ull, hit_hi = 0ull;
        {
            const float4 hi = S.posh[lane], li = S.posl[lane];
            const float delta = v.nb_delta;
            for (int k0 = 0; k0 < nn; k0 += 4) {
                int jj[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int k = k0 + q;
                    jj[q] = k < nn ? (int)((unsigned)(k < nei_rows ? nei_s[k * 32] : __ldg(&nei[(size_t)k * n + i])) & rmask)
                                   : -1;
                }
                float4 hj[4];
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (jj[q] >= 0) hj[q] = __ldg(&Aposh[jj[q]]);
                unsigned hit = 0u;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    if (jj[q] < 0) continue;
                    const int h = contact_hint(hi, hj[q], delta, per);
                    if (h > 0 || (h < 0 && exact_contact(hi, li, hj[q], __ldg(&Aposl[jj[q]]), per))) hit |= 1u << q;
                }
                if (k0 < 64)
                    hit_lo |= (unsigned long long)hit << k0;
                else
                    hit_hi |= (unsigned long long)hit << (k0 - 64);
            }
        }
        // ---- contacts through the ring: each round every lane queues its
        // next (up to) Q contacts in row order (partner and history slot);
        // whenever 32 are queued, or none will follow, the warp computes the
        // oldest 32 with every lane busy, and each lane adds its own results
        // in queue order, which is its row order
        int head = 0, tail = 0;
        while (true) {
            static_assert(Q == 2, "a lane queues at most two contacts per round");
            int cnt = 0;
            int qj0 = 0, qs0 = 0, qj1 = 0, qs1 = 0;
#pragma unroll 1
            for (int q = 0; q < Q && (hit_lo | hit_hi) != 0ull; q++) {
                int k;
                if (hit_lo) {
                    k = __ffsll((long long)hit_lo) - 1;
                    hit_lo &= hit_lo - 1ull;
                } else {
                    k = 64 + __ffsll((long long)hit_hi) - 1;
                    hit_hi &= hit_hi - 1ull;
                }
                const unsigned e = (unsigned)(k < nei_rows ? nei_s[k * 32] : __ldg(&nei[(size_t)k * n + i]));
                const int j = (int)(e & rmask);
                // the slot hint of the inner row, checked against the key
                const int hint = rmask != 0xFFFFFFFFu ? (int)(e >> kHintShift) - 1 : -1;
                bool fresh = false;
                int slot;
                if (hint >= 0 && hint < nc && P.hid[(size_t)hint * n + i] == j) {
                    slot = hint;
                } else {
                    slot = find_slot<Mixed>(P.hid, n, i, nc, j, v.hist_cap, fresh);
                    if (slot < 0) {
                        err |= 0x4u;
                        continue;
                    }
                    if (fresh) P.hid[(size_t)slot * n + i] = j;
                    if (rmask != 0xFFFFFFFFu && slot < 63) v.nei[(size_t)k * n + i] = j | ((slot + 1) << kHintShift);
                }
                touched |= 1ull << slot;
                if (cnt == 0) {
                    qj0 = j;
                    qs0 = slot | (fresh ? 64 : 0) | (lane << 7);
                } else {
                    qj1 = j;
                    qs1 = slot | (fresh ? 64 : 0) | (lane << 7);
                }
                cnt++;
            }
            int excl = cnt;
#pragma unroll
            for (int o2 = 1; o2 < 32; o2 <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, excl, o2);
                if (lane >= o2) excl += y;
            }
            const int added = __shfl_sync(0xffffffffu, excl, 31);
            excl -= cnt;
            if (cnt > 0) {
                const int x = (tail + excl) % kRing;
                que->j[x] = qj0;
                que->pk[x] = qs0;
            }
            if (cnt > 1) {
                const int x = (tail + excl + 1) % kRing;
                que->j[x] = qj1;
                que->pk[x] = qs1;
            }
            tail += added;
            const bool more = __any_sync(0xffffffffu, (hit_lo | hit_hi) != 0ull);
            while (tail - head >= 32 || (!more && tail > head)) {
                const int B = min(32, tail - head);
                que->owned[lane] = 0u;
                __syncwarp();
                // ---- the warp computes the batch [head, head + B)
                const int x = (head + lane) % kRing;
                const int sl = lane < B ? que->pk[x] : 0;
                const int ow = lane < B ? sl >> 7 : 32 + lane;
                if (lane < B) {
                    const int j = que->j[x];
                    const int slot = sl & 63;
                    const int iow = t * 32 + ow;
                    const float4 hiw = S.posh[ow], liw = S.posl[ow], viw = S.vel[ow], wiw = S.rot[ow];
                    const float4 hjq = __ldg(&Aposh[j]), ljq = __ldg(&Aposl[j]);
                    const float4 vj = __ldg(&Avel[j]), wj = __ldg(&Arot[j]);
                    const size_t h = (size_t)slot * n + iow;
                    Vec3<R> sp, cp;
                    if (sl & 64) {
                        sp.x = sp.y = sp.z = 0.f;
                        cp.x = cp.y = cp.z = 0.f;
                    } else {
                        sp.x = P.hx[h]; sp.y = P.hy[h]; sp.z = P.hz[h];
                        cp.x = P.cx[h]; cp.y = P.cy[h]; cp.z = P.cz[h];
                    }
                    const Mat mo = own_material<MODEL>(v, P, iow, hiw.w, viw.w);
                    const Force6 G = pair_force<MODEL>(v, pair_geometry(hiw, liw, hjq, ljq, per), hiw.w, hjq.w, viw,
                                                       wiw, vj, wj, viw.w, mo, sp, cp);
                    P.hx[h] = sp.x; P.hy[h] = sp.y; P.hz[h] = sp.z;
                    P.cx[h] = cp.x; P.cy[h] = cp.y; P.cz[h] = cp.z;
                    que->f[0][lane] = G.fx;
                    que->f[1][lane] = G.fy;
                    que->f[2][lane] = G.fz;
                    que->f[3][lane] = G.mx;
                    que->f[4][lane] = G.my;
                    que->f[5][lane] = G.mz;
                }
                // the batch positions of each owner: one mask per group of
                // equal owners, written by the group's first lane
                const unsigned grp = __match_any_sync(0xffffffffu, ow);
                if (lane < B && (grp & ((1u << lane) - 1u)) == 0u) que->owned[ow] = grp;
                __syncwarp();
                // each lane adds its own results in position (row) order
                for (unsigned m = que->owned[lane]; m != 0u; m &= m - 1u) {
                    const int y = __ffs((int)m) - 1;
                    F.fx += que->f[0][y];
                    F.fy += que->f[1][y];
                    F.fz += que->f[2][y];
                    F.mx += que->f[3][y];
                    F.my += que->f[4][y];
                    F.mz += que->f[5][y];
                }
                __syncwarp();
                head += B;
            }
            if (!more) break;
        }
        // ---- wall contacts, the geometry over the whole warp
        coop_walls<MODEL, WCAP, PER>(v, P, S, que, t, lane, active, active ? S.nneiw[lane] : 0, S.ncw[lane], F, err);
        if (active) {
            const Mat mt = own_material<MODEL>(v, P, i, S.posh[lane].w, S.vel[lane].w);
            P.nc[i] = surviving(touched, nc);
            Own o;
            o.wi = S.rot[lane];
            o.hi = S.posh[lane];
            o.li = S.posl[lane];
            o.vi = S.vel[lane];
            o.vl = __ldg(&A.vell[i]);
            o.wl = __ldg(&A.rotl[i]);
            o.rh = __ldg(&v.refh[i]);
            integrate_one<PER>(v, B, i, o, mt.invmoi, F, votes, err);
        }
        __syncwarp();
    }
    if (timed_out) {
        err |= 0x80u;
        // let the copies still in flight land before the shared memory goes away
        if (lane == 0) {
            mbar_wait_bounded(&full[warp][t_it & 1], (unsigned)(t_it >> 1) & 1u);
            if (t_next < nsub) mbar_wait_bounded(&full[warp][(t_it + 1) & 1], (unsigned)((t_it + 1) >> 1) & 1u);
        }
        __syncwarp();
    }
    step_epilogue(ctl, s, votes, err, cond, cond_inner, use_cond);
}

namespace {
// MINB: resident CTAs per SM a kernel's register allocation is sized for
// (cooperative kernel 4, 5 or 6; one-pass kernel 2 or 3).
// PER: compiled for a periodic x; those kernels exist for the default
// occupancy only (5 for the cooperative kernel, 2 for the one-pass kernel).
template <int MODEL, int MINB, bool PER>
void* direct_kernel_minb(int wall_cap) {
    if (wall_cap <= 16) return (void*)k_step_mixed<MODEL, 16, MINB, PER>;
    if (wall_cap <= 32) return (void*)k_step_mixed<MODEL, 32, MINB, PER>;
    return (void*)k_step_mixed<MODEL, 64, MINB, PER>;
}
template <int MODEL>
void* direct_kernel(int wall_cap, int minb, bool per) {
    if (per) return direct_kernel_minb<MODEL, 2, true>(wall_cap);
    return minb == 3 ? direct_kernel_minb<MODEL, 3, false>(wall_cap) : direct_kernel_minb<MODEL, 2, false>(wall_cap);
}
template <int MODEL, bool PER>
void* wtma_kernel(int wall_cap) {
    void* fn = wall_cap <= 16   ? (void*)k_step_mixed_wtma<MODEL, 16, PER>
               : wall_cap <= 32 ? (void*)k_step_mixed_wtma<MODEL, 32, PER>
                                : (void*)k_step_mixed_wtma<MODEL, 64, PER>;
    static bool configured[3] = {false, false, false};
    const int slot = wall_cap <= 16 ? 0 : (wall_cap <= 32 ? 1 : 2);
    if (!configured[slot]) {
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * kWarps * kWStageBytes);
        configured[slot] = true;
    }
    return fn;
}
template <int MODEL, int MINB, bool PER>
void* coop_kernel_minb(int wall_cap) {
    void* fn = wall_cap <= 16   ? (void*)k_step_mixed_coop<MODEL, 16, MINB, PER>
               : wall_cap <= 32 ? (void*)k_step_mixed_coop<MODEL, 32, MINB, PER>
                                : (void*)k_step_mixed_coop<MODEL, 64, MINB, PER>;
    static bool configured[3] = {false, false, false};
    const int slot = wall_cap <= 16 ? 0 : (wall_cap <= 32 ? 1 : 2);
    if (!configured[slot]) {
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCoopSmem);
        configured[slot] = true;
    }
    return fn;
}
template <int MODEL>
void* coop_kernel(int wall_cap, int minb, bool per) {
    if (per) return coop_kernel_minb<MODEL, 5, true>(wall_cap);
    return minb == 4 ? coop_kernel_minb<MODEL, 4, false>(wall_cap)
                     : (minb == 6 ? coop_kernel_minb<MODEL, 6, false>(wall_cap)
                                  : coop_kernel_minb<MODEL, 5, false>(wall_cap));
}
// Kernel and occupancy: the engine's settings, else the environment
// (GDEM_MIXED_KERNEL=staged|direct, GDEM_COOP_MINB, GDEM_MIXED_MINB), else the
// defaults (warp-cooperative, 5 CTAs per SM).
int env_int(const char* name, int dflt) {
    const char* e = getenv(name);
    return e ? atoi(e) : dflt;
}
int kernel_kind(const View<Mixed>& v) {
    if (v.kernel_variant > 0) return v.kernel_variant - 1;
    static const int k = [] {
        const char* e = getenv("GDEM_MIXED_KERNEL");
        if (e && strcmp(e, "direct") == 0) return 2;
        if (e && strcmp(e, "staged") == 0) return 1;
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

StepLaunch step_launch(const View<Mixed>& v, int reserve) {
    const int ntiles = (v.n + kBlock - 1) / kBlock;
    const int kind = kernel_kind(v);
    if (kind == 0) {
        static const int env_minb = env_int("GDEM_COOP_MINB", 5);
        const int minb = v.occupancy > 0 ? v.occupancy : env_minb;
        const bool per = v.per_x != 0;
        void* fn = v.mat.model == 1 ? coop_kernel<1>(v.wall_cap, minb, per) : coop_kernel<0>(v.wall_cap, minb, per);
        const size_t smem = kCoopSmem;
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kCoopWarps * 32, smem);
        if (per_sm < 1) per_sm = 1;
        const int nsub = (v.n + 31) / 32;
        const int need = (nsub + kCoopWarps - 1) / kCoopWarps;
        // GDEM_COOP_RESERVE overrides a nonzero reserve (tuning)
        static const int env_reserve = env_int("GDEM_COOP_RESERVE", -1);
        const int res = reserve > 0 && env_reserve >= 0 ? env_reserve : reserve;
        const int full = per_sm * sm_count() - res > 1 ? per_sm * sm_count() - res : 1;
        const int grid = need < full ? need : full;
        return StepLaunch{fn, dim3(grid), dim3(kCoopWarps * 32), smem};
    }
    if (kind == 1) {
        void* fn = v.per_x ? (v.mat.model == 1 ? wtma_kernel<1, true>(v.wall_cap) : wtma_kernel<0, true>(v.wall_cap))
                           : (v.mat.model == 1 ? wtma_kernel<1, false>(v.wall_cap) : wtma_kernel<0, false>(v.wall_cap));
        const int nsub = (v.n + 31) / 32;
        const int need = (nsub + kWarps - 1) / kWarps;
        const int grid = need < 2 * sm_count() ? need : 2 * sm_count();
        return StepLaunch{fn, dim3(grid), dim3(kBlock), (size_t)2 * kWarps * kWStageBytes};
    }
    static const int env_minb = env_int("GDEM_MIXED_MINB", 2);
    const int minb = v.occupancy > 0 ? v.occupancy : env_minb;
    const bool per = v.per_x != 0;
    void* fn = v.mat.model == 1 ? direct_kernel<1>(v.wall_cap, minb, per) : direct_kernel<0>(v.wall_cap, minb, per);
    return StepLaunch{fn, dim3(ntiles), dim3(kBlock), 0};
}

void launch_step(const View<Mixed>& v, cudaStream_t st, cudaGraphConditionalHandle cond, int use_cond) {
    const StepLaunch L = step_launch(v);
    View<Mixed> vv = v;
    cudaGraphConditionalHandle ci = cond;
    void* args[4] = {(void*)&vv, (void*)&cond, (void*)&ci, (void*)&use_cond};
    cudaLaunchKernel(L.fn, L.grid, L.block, args, L.smem, st);
}

}  // namespace gdem
