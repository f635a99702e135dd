// pmgb_img.cuh -- device code of the image-list Widom unit (see csrc/pmgb_img.cu), shared by the
// single-system kernel and the persistent batch kernel.
#pragma once
#include "pmgb_device.cuh"

namespace {

constexpr int kImgWarps = PMGB_THREADS / 32;
constexpr float kFarAway = 1.0e15f;               // padding image: r^2 ~ 1e30, beyond every cutoff

// Hilbert-curve cell (2^bits per axis) of Widom insertion idx: the key of the spatial order over a
// whole run.  The cell holds the insertion's centre of mass (the top bits of the first Philox draw
// of make_pose); along the curve a CTA's 256 insertions stay compact, and so does its list.
__device__ __forceinline__ int run_cell(unsigned long long seed, unsigned long long idx, int bits) {
    const uint2 key = make_uint2(static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    const uint4 a = philox4x32_10(make_uint4(static_cast<uint32_t>(idx), static_cast<uint32_t>(idx >> 32), 0u, 0u), key);
    return hilbert_cell(a.x >> (32 - bits), a.y >> (32 - bits), a.z >> (32 - bits), bits);
}

// Exclusive scan of n_cells counts (a multiple of 512) by one CTA of 1024 threads: chunks of
// 8192 consecutive cells, 8 per thread (two coalesced 16-byte loads), each chunk scanned by the
// CTA and offset by the running total.
__device__ __forceinline__ void scan_cells(int* counts, int n_cells) {
    __shared__ int wsum[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    int carry = 0;
    for (int base = 0; base < n_cells; base += 8192) {
        const int i0 = base + 8 * t;
        int v[8];
        if (i0 < n_cells) {
            const int4 a = *reinterpret_cast<const int4*>(counts + i0);
            const int4 b = *reinterpret_cast<const int4*>(counts + i0 + 4);
            v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
        } else {
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = 0;
        }
        int own = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) own += v[q];
        int incl = own;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) wsum[w] = incl;
        __syncthreads();
        if (w == 0) {
            int sum = wsum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, sum, o);
                if (lane >= o) sum += u;
            }
            wsum[lane] = sum;  // inclusive over warps
        }
        __syncthreads();
        int run = carry + (w > 0 ? wsum[w - 1] : 0) + incl - own;
        if (i0 < n_cells) {
            int4 a, b;
            a.x = run; run += v[0]; a.y = run; run += v[1]; a.z = run; run += v[2]; a.w = run; run += v[3];
            b.x = run; run += v[4]; b.y = run; run += v[5]; b.z = run; run += v[6]; b.w = run;
            *reinterpret_cast<int4*>(counts + i0) = a;
            *reinterpret_cast<int4*>(counts + i0 + 4) = b;
        }
        carry += wsum[31];
        __syncthreads();  // wsum is rewritten by the next chunk
    }
}

// ---- the image-list unit -------------------------------------------------------------------
// The CTA's list, per pair of images (32 + 32 bytes): {x0, x1, y0, y1}, {z0, z1, q0, q1} (FP32
// offsets from the CTA's centre, and charges) and {xl0, xl1, yl0, yl1}, {zl0, zl1, -, -} (the
// offsets' FP32 residuals: x + xl is the minimum-image offset to ~1e-13 A).
constexpr int kImgCap = 2048;                     // images in the CTA's list
constexpr float kImgClose2 = 16.0f;               // r^2 (A^2) below which the residuals are applied
constexpr size_t kImgListBytes = size_t(kImgCap) * 32;                            // 64 KB
constexpr size_t kImgSiteBytes = size_t(PMGB_THREADS) * 3 * 3 * sizeof(float);  // site residuals (<= 3 sites)
struct ImgScratch {
    uint32_t p0[3];                    // the CTA's reference position (fixed point)
    int mn[kImgWarps][3], mx[kImgWarps][3];
    uint32_t rho[kImgWarps];           // per warp, float bits (non-negative)
    int wsum[kImgWarps];               // per warp, images of the current pass
};
constexpr size_t kImgScratchBytes = (sizeof(ImgScratch) + 15) & ~size_t(15);
constexpr size_t kImgSmemBytes = kImgListBytes + kImgSiteBytes + kImgScratchBytes;

// FP32 Cartesian offset (h + p) . f of a fractional displacement f in fixed-point units
__device__ __forceinline__ void cart3(const SysDev& S, float fx, float fy, float fz, float& x, float& y, float& z) {
    x = __fadd_rn(fmaf(S.h00, fx, fmaf(S.h01, fy, __fmul_rn(S.h02, fz))),
                  fmaf(S.p00, fx, fmaf(S.p01, fy, __fmul_rn(S.p02, fz))));
    y = __fadd_rn(fmaf(S.h11, fy, __fmul_rn(S.h12, fz)), fmaf(S.p11, fy, __fmul_rn(S.p12, fz)));
    z = fmaf(S.h22, fz, __fmul_rn(S.p22, fz));
}

// Double-float Cartesian offset (h + p) . D of the fractional displacement D = d + n 2^32 in
// fixed-point units (d a 32-bit displacement, n a shift by whole cells): D splits exactly into a
// multiple of 4096 (d rounded down to one, plus n 2^32: at most 23 significant bits) and a
// remainder below 4096, both exact FP32 values; the products of the box matrix's FP32 value h
// with the first are exact (TwoProd), the rest are small corrections.  hi + lo is the FP64 product
// to ~1e-13 relative.  Every operation is explicit (no contraction left to the compiler, no 64-bit
// conversion), so that the lists, and the sums over them, are the same in every kernel that inlines
// this code.
__device__ __forceinline__ void df_mul_add(float h, float p, float dh, float dl, float& s, float& c) {
    // s + c += (h + p) (dh + dl), s the running FP32 sum of the exact products, c the corrections
    const float m = __fmul_rn(h, dh);
    const float e = fmaf(h, dh, -m);                       // h dh = m + e exactly
    const float t = __fadd_rn(s, m);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(m, bp));  // TwoSum
    s = t;
    c = __fadd_rn(c, __fadd_rn(__fadd_rn(err, e), fmaf(h, dl, __fmul_rn(p, dh))));
}

__device__ __forceinline__ void cart_df(const SysDev& S, const int d[3], const int n[3], float& x, float& y, float& z,
                                        float& xl, float& yl, float& zl) {
    float dh[3], dl[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        dh[a] = __fadd_rn(__int2float_rn(d[a] & ~0xFFF), __fmul_rn(static_cast<float>(n[a]), 4294967296.0f));
        dl[a] = __int2float_rn(d[a] & 0xFFF);
    }
    float s = 0.0f, c = 0.0f;
    df_mul_add(S.h00, S.p00, dh[0], dl[0], s, c);
    df_mul_add(S.h01, S.p01, dh[1], dl[1], s, c);
    df_mul_add(S.h02, S.p02, dh[2], dl[2], s, c);
    x = __fadd_rn(s, c);
    xl = __fsub_rn(c, __fsub_rn(x, s));
    s = c = 0.0f;
    df_mul_add(S.h11, S.p11, dh[1], dl[1], s, c);
    df_mul_add(S.h12, S.p12, dh[2], dl[2], s, c);
    y = __fadd_rn(s, c);
    yl = __fsub_rn(c, __fsub_rn(y, s));
    s = c = 0.0f;
    df_mul_add(S.h22, S.p22, dh[2], dl[2], s, c);
    z = __fadd_rn(s, c);
    zl = __fsub_rn(c, __fsub_rn(z, s));
}

// One Widom insertion per thread; the CTA builds one list for its 256 insertions (the records
// are read once per CTA, each thread taking one record per pass) and every warp evaluates its
// lanes against it.  smem: kImgSmemBytes (list, the threads' site residuals, scratch).
// COLS: also the adjoint's columns, per (species segment, site) the sums of r^-12 and r^-6 within
// the LJ cutoff, into io.dsum[((sg NS + k) 2 + {0, 1}) io.dsum_stride + io.col_item].
template <int NS, bool CHARGED, bool STATS, bool COLS = false>
__device__ __forceinline__ void img_unit(const SysDev& S, const UnitIO& io, unsigned char* smem) {
    static_assert(NS <= 3, "site residuals are kept for three sites");
    const unsigned full = 0xffffffffu;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool valid = io.valid;
    const long long item = io.item;
    float4* list = reinterpret_cast<float4*>(smem);
    float* wf = reinterpret_cast<float*>(smem);
    float* site_lo = reinterpret_cast<float*>(smem + kImgListBytes) + tid * 9;
    ImgScratch& sc = *reinterpret_cast<ImgScratch*>(smem + kImgListBytes + kImgSiteBytes);

    uint32_t ux[NS], uy[NS], uz[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) ux[k] = uy[k] = uz[k] = 0u;
    bool blocked = false;
    if (valid) {
        float com[3];
        pose_sites<NS>(S, io.seed, static_cast<unsigned long long>(item), ux, uy, uz, com);
        if (S.acc) blocked = !accessible_com(S, com);
    }
    const bool active = valid && !blocked;

    // reciprocal space from the fixed-point sites (before they are replaced by offsets)
    float pl_hi = 0.0f, pl_lo = 0.0f;
    if (CHARGED && valid) kspace_fwd<NS, false>(S, ux, uy, uz, pl_hi, pl_lo);

    // ---- the CTA's centre and reach ----
    // reference: thread 0's first site (thread 0 holds an insertion in every unit that has one)
    if (tid == 0) {
        sc.p0[0] = ux[0];
        sc.p0[1] = uy[0];
        sc.p0[2] = uz[0];
    }
    __syncthreads();
    const uint32_t p0[3] = {sc.p0[0], sc.p0[1], sc.p0[2]};
    {
        int mn[3] = {INT_MAX, INT_MAX, INT_MAX}, mx[3] = {INT_MIN, INT_MIN, INT_MIN};
        if (active) {
#pragma unroll
            for (int k = 0; k < NS; ++k)
                if (k < S.n_sites) {
                    const int d[3] = {static_cast<int>(ux[k] - p0[0]), static_cast<int>(uy[k] - p0[1]),
                                      static_cast<int>(uz[k] - p0[2])};
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        mn[a] = min(mn[a], d[a]);
                        mx[a] = max(mx[a], d[a]);
                    }
                }
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            mn[a] = __reduce_min_sync(full, mn[a]);
            mx[a] = __reduce_max_sync(full, mx[a]);
            if (lane == 0) {
                sc.mn[warp][a] = mn[a];
                sc.mx[warp][a] = mx[a];
            }
        }
    }
    __syncthreads();
    uint32_t c[3];
    bool any_active = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int lo = INT_MAX, hi = INT_MIN;
        for (int w = 0; w < kImgWarps; ++w) {
            lo = min(lo, sc.mn[w][a]);
            hi = max(hi, sc.mx[w][a]);
        }
        any_active = lo <= hi;  // the same on every axis
        c[a] = p0[a] + static_cast<uint32_t>(static_cast<int>((static_cast<long long>(lo) + hi) >> 1));
    }
    // the sites' negated Cartesian offsets from c (FP32, residuals in shared memory) and the reach rho
    float nx[NS], ny[NS], nz[NS];
    {
        float rho = 0.0f;
#pragma unroll
        for (int k = 0; k < NS; ++k) {
            const int D[3] = {static_cast<int>(ux[k] - c[0]), static_cast<int>(uy[k] - c[1]),
                              static_cast<int>(uz[k] - c[2])};
            const int n0[3] = {0, 0, 0};
            float x, y, z, xl, yl, zl;
            cart_df(S, D, n0, x, y, z, xl, yl, zl);
            nx[k] = -x;
            ny[k] = -y;
            nz[k] = -z;
            site_lo[3 * k + 0] = -xl;
            site_lo[3 * k + 1] = -yl;
            site_lo[3 * k + 2] = -zl;
            if (active && k < S.n_sites) rho = fmaxf(rho, sqrtf(fmaf(x, x, fmaf(y, y, __fmul_rn(z, z)))));
        }
        const uint32_t rw = __reduce_max_sync(full, __float_as_uint(rho));  // non-negative floats
        if (lane == 0) sc.rho[warp] = rw;
    }
    __syncthreads();
    uint32_t rmax = 0u;
    for (int w = 0; w < kImgWarps; ++w) rmax = max(rmax, sc.rho[w]);
    const float rho = __uint_as_float(rmax);

    float lj_hi[NS], lj_lo[NS], ph_hi[NS], ph_lo[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) lj_hi[k] = lj_lo[k] = ph_hi[k] = ph_lo[k] = 0.0f;
    bool ovl = false;
    unsigned long long st_dist = 0, st_lj = 0, st_es = 0;
    if (any_active) {  // uniform over the CTA
        const float reach = fmaf(__fadd_rn(sqrtf(fmaxf(S.rc2, CHARGED ? S.rc2e : 0.0f)), rho), 1.00001f, 1e-4f);
        const float reach2 = __fmul_rn(reach, reach);
        // reach as a fraction of each perpendicular width: the image d + n (fractions of the
        // supercell) of a record can lie within reach of c only if |d_a + n_a| < t_a on every axis;
        // a record has at most g_a shifts along axis a, so a pass of n_pass records adds at most
        // n_pass g_0 g_1 g_2 <= kImgCap images
        float t[3];
        int g = 1;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            t[a] = __fdiv_rn(reach, __fmul_rn(S.cw[a], 4294967296.0f));
            g *= static_cast<int>(floorf(__fadd_rn(__fmul_rn(2.0f, t[a]), 2e-6f))) + 1;
        }
        const int n_pass = max(1, min(PMGB_THREADS, kImgCap / g));

        const Geo2 g2{f2(S.h00), f2(S.h01), f2(S.h02), f2(S.h11), f2(S.h12), f2(S.h22),
                      f2(S.p00), f2(S.p01), f2(S.p02), f2(S.p11), f2(S.p12), f2(S.p22),
                      S.rc2, S.rc2e, fmaxf(S.rc2, CHARGED ? S.rc2e : 0.0f), f2(0.5f * S.alpha),
                      f2(-S.alpha * S.alpha * 1.4426950408889634f)};

        for (int sg = 0; sg < S.n_seg; ++sg) {
            const SegDesc dsc = S.seg[sg];
            float segmin[NS], lj12[NS], lj6[NS];
            float2 i12[NS], i6[NS];  // COLS: the segment's column sums
#pragma unroll
            for (int k = 0; k < NS; ++k) {
                const SitePar p = S.segpar[sg * PMGB_MAX_SITES + k];
                lj12[k] = p.lj12;
                lj6[k] = p.lj6;
                segmin[k] = __int_as_float(0x7f800000);
                i12[k] = i6[k] = f2(0.0f);
            }
            int n = 0;  // images in the list (the same in every thread)
            // evaluate the list (padded to whole groups of four) in every warp, and empty it
            auto flush = [&]() {
                const int n4 = (n + 3) & ~3;
                if (tid < n4 - n) {
                    const int i = n + tid, q = i >> 1, h = i & 1;
                    wf[q * 16 + 0 + h] = kFarAway;
#pragma unroll
                    for (int f = 2; f < 14; f += 2) wf[q * 16 + f + h] = 0.0f;
                }
                __syncthreads();
                if (STATS && active) st_dist += static_cast<unsigned long long>(n) * S.n_sites;
                float2 ljp2[NS], php2[NS];
#pragma unroll
                for (int k = 0; k < NS; ++k) ljp2[k] = php2[k] = f2(0.0f);
                for (int i = 0; i < n4; i += 4) {
                    const float4* P0 = list + (i >> 1) * 4;  // pair i/2: A, B, C, D; pair i/2 + 1 follows
                    const float4 A0 = P0[0], B0 = P0[1], A1 = P0[4], B1 = P0[5];
                    // the distances of every site first, one vote for the group, then the terms of
                    // every site: 2 NS independent chains (sites of a guest are near or far together)
                    float2 d01[NS], d23[NS];
                    float m01 = __int_as_float(0x7f800000), m23 = m01;
#pragma unroll
                    for (int k = 0; k < NS; ++k) {
                        const float2 sx = f2(nx[k]), sy = f2(ny[k]), sz = f2(nz[k]);
                        const float2 ex0 = __fadd2_rn(make_float2(A0.x, A0.y), sx);
                        const float2 ey0 = __fadd2_rn(make_float2(A0.z, A0.w), sy);
                        const float2 ez0 = __fadd2_rn(make_float2(B0.x, B0.y), sz);
                        const float2 ex1 = __fadd2_rn(make_float2(A1.x, A1.y), sx);
                        const float2 ey1 = __fadd2_rn(make_float2(A1.z, A1.w), sy);
                        const float2 ez1 = __fadd2_rn(make_float2(B1.x, B1.y), sz);
                        d01[k] = fma2(ex0, ex0, fma2(ey0, ey0, mul2(ez0, ez0)));
                        d23[k] = fma2(ex1, ex1, fma2(ey1, ey1, mul2(ez1, ez1)));
                        if (k < S.n_sites) {
                            m01 = fminf(m01, fminf(d01[k].x, d01[k].y));
                            m23 = fminf(m23, fminf(d23[k].x, d23[k].y));
                        }
                    }
                    // one vote per pair of images: bits 0, 1 some lane reaches images 0-1, 2-3;
                    // bits 2, 3 some lane has a pair there within the residuals' radius
                    // (uncharged: the LJ terms are cheap, one vote for the group costs less)
                    const float mg = fminf(m01, m23);
                    const unsigned flags = __reduce_or_sync(
                        full, !active ? 0u
                              : CHARGED ? (unsigned(m01 < g2.rcmax2) | unsigned(m23 < g2.rcmax2) << 1 |
                                           unsigned(m01 < kImgClose2) << 2 | unsigned(m23 < kImgClose2) << 3)
                                        : (unsigned(mg < g2.rcmax2) * 3u | unsigned(mg < kImgClose2) * 12u));
                    if (flags & 3u) {
                        if (flags & 12u) {
                            // close pairs: r^2 = |e + delta|^2 with delta = the offsets' residuals
                            // (|delta| ~ 1e-6 A): add 2 e . delta
                            const float4 C0 = P0[2], D0 = P0[3], C1 = P0[6], D1 = P0[7];
#pragma unroll
                            for (int k = 0; k < NS; ++k) {
                                const float2 sx = f2(nx[k]), sy = f2(ny[k]), sz = f2(nz[k]);
                                const float2 lx = f2(site_lo[3 * k + 0]), ly = f2(site_lo[3 * k + 1]),
                                             lz = f2(site_lo[3 * k + 2]);
                                const float2 ex0 = __fadd2_rn(make_float2(A0.x, A0.y), sx);
                                const float2 ey0 = __fadd2_rn(make_float2(A0.z, A0.w), sy);
                                const float2 ez0 = __fadd2_rn(make_float2(B0.x, B0.y), sz);
                                const float2 ex1 = __fadd2_rn(make_float2(A1.x, A1.y), sx);
                                const float2 ey1 = __fadd2_rn(make_float2(A1.z, A1.w), sy);
                                const float2 ez1 = __fadd2_rn(make_float2(B1.x, B1.y), sz);
                                const float2 dx0 = __fadd2_rn(make_float2(C0.x, C0.y), lx);
                                const float2 dy0 = __fadd2_rn(make_float2(C0.z, C0.w), ly);
                                const float2 dz0 = __fadd2_rn(make_float2(D0.x, D0.y), lz);
                                const float2 dx1 = __fadd2_rn(make_float2(C1.x, C1.y), lx);
                                const float2 dy1 = __fadd2_rn(make_float2(C1.z, C1.w), ly);
                                const float2 dz1 = __fadd2_rn(make_float2(D1.x, D1.y), lz);
                                d01[k] = fma2(f2(2.0f), fma2(ex0, dx0, fma2(ey0, dy0, mul2(ez0, dz0))), d01[k]);
                                d23[k] = fma2(f2(2.0f), fma2(ex1, dx1, fma2(ey1, dy1, mul2(ez1, dz1))), d23[k]);
                                // overlaps (r^2 < R^2_overlap = 0.1 A^2, far inside the close radius)
                                // can only occur in a group that raised the close vote
                                if (k < S.n_sites)
                                    segmin[k] = fminf(segmin[k], fminf(fminf(d01[k].x, d01[k].y), fminf(d23[k].x, d23[k].y)));
                            }
                        }
                        // the terms of the reached pairs (those of the others are exact zeros); both
                        // pairs together where both are reached, for 2 NS independent chains.  Every
                        // one of the NS sites, with no branch between them: the terms of a padding
                        // site (k >= n_sites) go to sums that are never read
                        if ((flags & 3u) == 3u) {
#pragma unroll
                            for (int k = 0; k < NS; ++k) {
                                const float2 a12 = f2(lj12[k]), a6 = f2(lj6[k]);
                                pair2_energy<CHARGED, COLS>(d01[k], B0.z, B0.w, g2, a12, a6, ljp2[k], php2[k], &i12[k], &i6[k]);
                                pair2_energy<CHARGED, COLS>(d23[k], B1.z, B1.w, g2, a12, a6, ljp2[k], php2[k], &i12[k], &i6[k]);
                            }
                        } else {
                            const bool first = flags & 1u;
                            const float qa = first ? B0.z : B1.z, qb = first ? B0.w : B1.w;
#pragma unroll
                            for (int k = 0; k < NS; ++k) {
                                const float2 a12 = f2(lj12[k]), a6 = f2(lj6[k]);
                                pair2_energy<CHARGED, COLS>(first ? d01[k] : d23[k], qa, qb, g2, a12, a6, ljp2[k], php2[k],
                                                            &i12[k], &i6[k]);
                            }
                        }
                    }
#pragma unroll
                    for (int k = 0; k < NS; ++k) {
                        if (k >= S.n_sites) continue;
                        if (STATS && active) {
                            st_lj += (d01[k].x < g2.rc2) + (d01[k].y < g2.rc2) + (d23[k].x < g2.rc2) + (d23[k].y < g2.rc2);
                            if (CHARGED)
                                st_es += (d01[k].x < g2.rc2e) + (d01[k].y < g2.rc2e) + (d23[k].x < g2.rc2e) +
                                         (d23[k].y < g2.rc2e);
                        }
                    }
                    if ((i & 63) == 60 || i + 4 >= n4) {  // compensated fold every 64 images
#pragma unroll
                        for (int k = 0; k < NS; ++k) {
                            two_sum_acc(lj_hi[k], lj_lo[k], __fadd_rn(ljp2[k].x, ljp2[k].y));
                            if (CHARGED) two_sum_acc(ph_hi[k], ph_lo[k], __fadd_rn(php2[k].x, php2[k].y));
                            ljp2[k] = php2[k] = f2(0.0f);
                        }
                    }
                }
                __syncthreads();  // every warp is done with the list before it is written again
                n = 0;
            };
            for (int base = dsc.lo; base < dsc.hi; base += n_pass) {
                // this thread's record of the pass and the cell shifts that can bring it within reach
                const int j = base + tid;
                const bool in = tid < n_pass && j < dsc.hi;
                const int4 r = in ? __ldg(S.rec + j) : make_int4(0, 0, 0, 0);
                int dd[3], lo[3], hi[3];
                float fd[3];
                const uint32_t rv[3] = {static_cast<uint32_t>(r.x), static_cast<uint32_t>(r.y), static_cast<uint32_t>(r.z)};
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const int d = static_cast<int>(rv[a] - c[a]);
                    dd[a] = d;
                    fd[a] = __int2float_rn(d);
                    const float df = __fmul_rn(fd[a], 2.3283064365386963e-10f);  // fraction in [-1/2, 1/2]
                    // the cell shifts n_a with |d_a + n_a| < t_a, widened by a rounding margin
                    lo[a] = in ? static_cast<int>(ceilf(__fsub_rn(__fsub_rn(-t[a], df), 1e-6f))) : 1;
                    hi[a] = in ? static_cast<int>(floorf(__fadd_rn(__fsub_rn(t[a], df), 1e-6f))) : 0;
                }
                // its images within reach: counted, then (after the CTA's scan) written
                auto images = [&](auto&& emit) {
                    for (int na = lo[0]; na <= hi[0]; ++na)
                        for (int nb = lo[1]; nb <= hi[1]; ++nb)
                            for (int nc = lo[2]; nc <= hi[2]; ++nc) {
                                // FP32 screen (reach carries a 1e-5 relative margin, far above its
                                // rounding); the double-float offset only for the images kept
                                float x, y, z;
                                cart3(S, __fadd_rn(fd[0], __fmul_rn(static_cast<float>(na), 4294967296.0f)),
                                      __fadd_rn(fd[1], __fmul_rn(static_cast<float>(nb), 4294967296.0f)),
                                      __fadd_rn(fd[2], __fmul_rn(static_cast<float>(nc), 4294967296.0f)), x, y, z);
                                if (fmaf(x, x, fmaf(y, y, __fmul_rn(z, z))) < reach2) emit(na, nb, nc);
                            }
                };
                int m = 0;
                images([&](int, int, int) { ++m; });
                // exclusive scan of the counts over the CTA
                int incl = m;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int v = __shfl_up_sync(full, incl, o);
                    if (lane >= o) incl += v;
                }
                if (lane == 31) sc.wsum[warp] = incl;
                __syncthreads();
                int before = 0, total = 0;
                for (int w = 0; w < kImgWarps; ++w) {
                    const int v = sc.wsum[w];
                    before += w < warp ? v : 0;
                    total += v;
                }
                if (n + total > kImgCap) flush();  // uniform: n and total are the CTA's
                int i = n + before + incl - m;
                images([&](int na, int nb, int nc) {
                    if (i >= kImgCap) return;  // cannot happen (n_pass g <= kImgCap); keeps writes in the list
                    const int nn[3] = {na, nb, nc};
                    float x, y, z, xl, yl, zl;
                    cart_df(S, dd, nn, x, y, z, xl, yl, zl);
                    const int q = i >> 1, h = i & 1;
                    wf[q * 16 + 0 + h] = x;
                    wf[q * 16 + 2 + h] = y;
                    wf[q * 16 + 4 + h] = z;
                    wf[q * 16 + 6 + h] = __int_as_float(r.w);
                    wf[q * 16 + 8 + h] = xl;
                    wf[q * 16 + 10 + h] = yl;
                    wf[q * 16 + 12 + h] = zl;
                    ++i;
                });
                n = min(n + total, kImgCap);
                __syncthreads();  // the pass's images are written; sc.wsum may be reused
            }
            if (n > 0) flush();
            if (COLS && valid) {
#pragma unroll
                for (int k = 0; k < NS; ++k) {
                    float* c12 = io.dsum + static_cast<size_t>((sg * NS + k) * 2) * io.dsum_stride + io.col_item;
                    c12[0] = __fadd_rn(i12[k].x, i12[k].y);
                    c12[io.dsum_stride] = __fadd_rn(i6[k].x, i6[k].y);
                }
            }
#pragma unroll
            for (int k = 0; k < NS; ++k)  // the overlap radii read again: no registers held over the loop
                ovl = ovl || (k < S.n_sites && segmin[k] < __ldg(&S.segpar[sg * PMGB_MAX_SITES + k].r2ovl));
        }
    }
    if (STATS) {
        unsigned long long cnt[3] = {st_dist, st_lj, st_es};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) cnt[i] += __shfl_xor_sync(full, cnt[i], o);
            if (lane == 0 && cnt[i]) atomicAdd(io.stats + i, cnt[i]);
        }
    }

    // ---- per-insertion energies (FP64), as run_unit forms them ----
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    double uv = 0.0, usr = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        if (k < S.n_sites) {
            uv = __dadd_rn(uv, __dadd_rn(static_cast<double>(lj_hi[k]), static_cast<double>(lj_lo[k])));
            if (CHARGED && S.q[k] != 0.0f)
                usr = fma(static_cast<double>(S.q[k]), __dadd_rn(static_cast<double>(ph_hi[k]), static_cast<double>(ph_lo[k])), usr);
        }
    }
    if (ovl) uv = inf;
    usr = __dmul_rn(usr, S.coul);
    const double ulr = CHARGED ? __dadd_rn(static_cast<double>(pl_hi), static_cast<double>(pl_lo)) : 0.0;
    double ues = __dadd_rn(usr, ulr);
    if (blocked) {  // src/henry.jl:230-233
        uv = inf;
        ues = inf;
    }
    if (valid) {
        io.u_out[2 * item + 0] = uv;
        io.u_out[2 * item + 1] = ues;
    }
}

}  // namespace
