// k_project.cu -- Fourier-slice projection of the padded 3D reference (or
// in-plane rotation of a padded 2D class reference) and the translation
// phase tables.
//
// Projection follows Projector::project (src/projector.cpp:630-733): the
// 2D frequency (x, y) is rotated by pad * A^-1 into the half volume, mirrored
// through the origin (complex conjugate) when the rotated x is negative, and
// interpolated trilinearly.  The reference GPU path uses hardware texture
// filtering (src/acc/acc_projector_impl.h:65-105), whose 8-bit fixed-point
// weights cannot hold the CPU's double result to 1e-5; this kernel
// interpolates in FP32 in software.  Each output pixel is independent; the
// 8 corners of a 3D sample are fetched through the texture path from a 3D
// CUDA array copy of the volume (point sampling: the stored values exactly;
// the array's blocked layout keeps a cell's corners and the cells of
// neighbouring pixels in few cache lines), or read from the linear volume.
#include "gbr_internal.h"

namespace gbr {

namespace {

__device__ __forceinline__ float2 lerp2(float a, float2 l, float2 h) {
    return make_float2(fmaf(h.x - l.x, a, l.x), fmaf(h.y - l.y, a, l.y));
}

// Trilinear sample of one class volume at 2D frequency (x, y) rotated by Ai.
// Returns false if the pixel lies outside r_max (value 0 then).
__device__ __forceinline__ float2 tex_at(cudaTextureObject_t t, int x, int y, int z) {
    return tex3D<float2>(t, (float)x + 0.5f, (float)y + 0.5f, (float)z + 0.5f);
}

__device__ __forceinline__ float2 sample_slice(const float2 *__restrict__ vol, const VolGeom g,
                                               const float *Ai, int x, int y, cudaTextureObject_t tex = 0) {
    // Inside-radius test in integers: |Ai (x,y,0)|^2 = pad^2 (x^2+y^2).
    const int rref = g.r_max * g.pad;
    if (g.pad * g.pad * (x * x + y * y) > rref * rref) return make_float2(0.f, 0.f);
    float xp = fmaf(Ai[0], (float)x, Ai[1] * (float)y);
    float yp = fmaf(Ai[3], (float)x, Ai[4] * (float)y);
    if (g.dim == 2) {
        // Projector::rotate2D (src/projector.cpp:1010-1100): bilinear in the
        // padded 2D reference, Friedel mate for negative x
        const bool neg2 = xp < 0.f;
        if (neg2) {
            xp = -xp;
            yp = -yp;
        }
        const float fx0 = floorf(xp), fy0 = floorf(yp);
        const float fx = xp - fx0, fy = yp - fy0;
        const int x0 = (int)fx0, y0 = (int)fy0 - g.yinit;
        if (x0 < 0 || x0 + 1 >= g.xdim || y0 < 0 || y0 + 1 >= g.ydim) return make_float2(0.f, 0.f);
        const float2 *b = vol + (size_t)y0 * g.xdim + x0;
        const float2 d00 = __ldg(b), d01 = __ldg(b + 1);
        const float2 d10 = __ldg(b + g.xdim), d11 = __ldg(b + g.xdim + 1);
        float2 v = lerp2(fy, lerp2(fx, d00, d01), lerp2(fx, d10, d11));
        if (neg2) v.y = -v.y;
        return v;
    }
    float zp = fmaf(Ai[6], (float)x, Ai[7] * (float)y);
    const bool neg = xp < 0.f;
    if (neg) {
        xp = -xp;
        yp = -yp;
        zp = -zp;
    }
    const float fx0 = floorf(xp), fy0 = floorf(yp), fz0 = floorf(zp);
    const float fx = xp - fx0, fy = yp - fy0, fz = zp - fz0;
    const int x0 = (int)fx0;
    const int y0 = (int)fy0 - g.yinit;
    const int z0 = (int)fz0 - g.zinit;
    if (x0 < 0 || x0 + 1 >= g.xdim || y0 < 0 || y0 + 1 >= g.ydim || z0 < 0 || z0 + 1 >= g.zdim)
        return make_float2(0.f, 0.f);
    float2 d000, d001, d010, d011, d100, d101, d110, d111;
    if (tex) {
        d000 = tex_at(tex, x0, y0, z0);
        d001 = tex_at(tex, x0 + 1, y0, z0);
        d010 = tex_at(tex, x0, y0 + 1, z0);
        d011 = tex_at(tex, x0 + 1, y0 + 1, z0);
        d100 = tex_at(tex, x0, y0, z0 + 1);
        d101 = tex_at(tex, x0 + 1, y0, z0 + 1);
        d110 = tex_at(tex, x0, y0 + 1, z0 + 1);
        d111 = tex_at(tex, x0 + 1, y0 + 1, z0 + 1);
    } else {
        const size_t sy = (size_t)g.xdim, sz = (size_t)g.xdim * g.ydim;
        const float2 *b = vol + (size_t)z0 * sz + (size_t)y0 * sy + x0;
        d000 = __ldg(b);
        d001 = __ldg(b + 1);
        d010 = __ldg(b + sy);
        d011 = __ldg(b + sy + 1);
        d100 = __ldg(b + sz);
        d101 = __ldg(b + sz + 1);
        d110 = __ldg(b + sz + sy);
        d111 = __ldg(b + sz + sy + 1);
    }
    const float2 dx00 = lerp2(fx, d000, d001);
    const float2 dx01 = lerp2(fx, d100, d101);
    const float2 dx10 = lerp2(fx, d010, d011);
    const float2 dx11 = lerp2(fx, d110, d111);
    const float2 dxy0 = lerp2(fy, dx00, dx10);
    const float2 dxy1 = lerp2(fy, dx01, dx11);
    float2 v = lerp2(fz, dxy0, dxy1);
    if (neg) v.y = -v.y;
    return v;
}

// circ[j] >= 0 marks the pixels exactly on the r_max circle; bit circ[j] of
// mask[orientation] says whether the reference projects it for that
// orientation (decided on the host in double precision as
// Projector::project does, src/projector.cpp:638-672).  Pixels with
// x^2 + y^2 > rout2 (rout2 >= 0) are not projected: the reference fills only
// the circle of the output image, radius XSIZE - 1 = size / 2 (:641-660,
// rotate2D :1020-1048), which for the coarse pass is smaller than r_max.
__global__ void k_project_rows(const float2 *const *__restrict__ vols, const VolGeom g,
                               const float *__restrict__ eul, const int *__restrict__ cls,
                               const int *__restrict__ orient_ids, int n_orient,
                               const PixelRef *__restrict__ pix, int npix, float *__restrict__ out_ri,
                               int ld, float *__restrict__ out_p2, int ld2, float2 *__restrict__ out_c,
                               const int *__restrict__ circ, const unsigned long long *__restrict__ mask,
                               int rout2, const unsigned long long *__restrict__ texs) {
    const int o = blockIdx.y;
    if (o >= n_orient) return;
    const int oid = orient_ids ? orient_ids[o] : o;
    __shared__ float Ai[9];
    if (threadIdx.x < 9) Ai[threadIdx.x] = eul[(size_t)oid * 9 + threadIdx.x];
    __syncthreads();
    const float2 *vol = vols[cls[oid]];
    const cudaTextureObject_t tex = (texs && g.dim == 3) ? (cudaTextureObject_t)texs[cls[oid]] : 0;
    const unsigned long long cm = mask ? mask[oid] : ~0ull;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < npix; j += gridDim.x * blockDim.x) {
        const PixelRef pr = pix[j];
        const int cb = circ ? circ[j] : -1;
        const bool outside = rout2 >= 0 && pr.x * pr.x + pr.y * pr.y > rout2;
        const float2 v = (outside || (cb >= 0 && !((cm >> cb) & 1ull))) ? make_float2(0.f, 0.f)
                                                                        : sample_slice(vol, g, Ai, pr.x, pr.y, tex);
        if (out_ri) {
            float *row = out_ri + (size_t)oid * ld;
            row[2 * j] = v.x;
            row[2 * j + 1] = v.y;
        }
        if (out_p2) out_p2[(size_t)oid * ld2 + j] = v.x * v.x + v.y * v.y;
        if (out_c) out_c[(size_t)oid * npix + j] = v;
    }
}

// e^{-2 pi i (x tx + y ty) / ori} in double, rounded to float
// (shiftImageInFourierTransform, src/fftw.cpp:842-920: zero shift is exact).
__global__ void k_phase_table(float2 *__restrict__ out, const double *__restrict__ tx,
                              const double *__restrict__ ty, int ntrans,
                              const PixelRef *__restrict__ pix, int npix, int ld, double ori) {
    const int t = blockIdx.y;
    if (t >= ntrans) return;
    const double xs = tx[t] / -ori, ys = ty[t] / -ori;
    const bool zero = fabs(xs) < 1e-6 && fabs(ys) < 1e-6;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < npix; j += gridDim.x * blockDim.x) {
        float2 e = make_float2(1.f, 0.f);
        if (!zero) {
            const double dotp = 2 * 3.14159265358979323846 * (pix[j].x * xs + pix[j].y * ys);
            double s, c;
            sincos(dotp, &s, &c);
            e = make_float2((float)c, (float)s);
        }
        out[(size_t)t * ld + j] = e;
    }
}

}  // namespace

cudaError_t vol_texture_update(VolTexture &t, const float2 *vol, const VolGeom &g, cudaStream_t st) {
    if (g.dim != 3) return cudaSuccess;
    cudaError_t e = cudaSuccess;
    if (!t.arr || t.x != g.xdim || t.y != g.ydim || t.z != g.zdim) {
        vol_texture_release(t);
        const cudaChannelFormatDesc fd = cudaCreateChannelDesc<float2>();
        e = cudaMalloc3DArray(&t.arr, &fd, make_cudaExtent(g.xdim, g.ydim, g.zdim));
        if (e != cudaSuccess) {
            t.arr = nullptr;
            return e;
        }
        t.x = g.xdim;
        t.y = g.ydim;
        t.z = g.zdim;
        cudaResourceDesc rd = {};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = t.arr;
        cudaTextureDesc td = {};
        td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
        td.filterMode = cudaFilterModePoint;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 0;
        e = cudaCreateTextureObject(&t.tex, &rd, &td, nullptr);
        if (e != cudaSuccess) return e;
    }
    cudaMemcpy3DParms cp = {};
    cp.srcPtr = make_cudaPitchedPtr(const_cast<float2 *>(vol), sizeof(float2) * g.xdim, g.xdim, g.ydim);
    cp.dstArray = t.arr;
    cp.extent = make_cudaExtent(g.xdim, g.ydim, g.zdim);
    cp.kind = cudaMemcpyDeviceToDevice;
    return cudaMemcpy3DAsync(&cp, st);
}

void vol_texture_release(VolTexture &t) {
    if (t.tex) cudaDestroyTextureObject(t.tex);
    if (t.arr) cudaFreeArray(t.arr);
    t = VolTexture();
}

cudaError_t launch_project_rows(const float2 *const *vols, const VolGeom &g, const float *eul,
                                const int *cls, const int *orient_ids, int n_orient,
                                const PixelRef *pix, int npix, float *out_ri, int ld, float *out_p2,
                                int ld2, float2 *out_c, cudaStream_t st, const int *circ,
                                const unsigned long long *mask, int rout2, const unsigned long long *texs) {
    if (n_orient <= 0 || npix <= 0) return cudaSuccess;
    const int threads = 128;
    const int bx = (npix + threads - 1) / threads;
    for (int o0 = 0; o0 < n_orient; o0 += 65535) {
        const int n = n_orient - o0 < 65535 ? n_orient - o0 : 65535;
        dim3 grid(bx, n);
        k_project_rows<<<grid, threads, 0, st>>>(vols, g, eul, cls, orient_ids ? orient_ids + o0 : nullptr,
                                                 n, pix, npix, out_ri ? out_ri + (orient_ids ? 0 : (size_t)o0 * ld) : nullptr,
                                                 ld, out_p2 ? out_p2 + (orient_ids ? 0 : (size_t)o0 * ld2) : nullptr,
                                                 ld2, out_c ? out_c + (orient_ids ? 0 : (size_t)o0 * npix) : nullptr,
                                                 circ, mask, rout2, texs);
        if (!orient_ids) {
            // rows are addressed by the orientation index; shift eul/cls/mask too
            eul += (size_t)n * 9;
            cls += n;
            if (mask) mask += n;
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_phase_table(float2 *out, const double *tx, const double *ty, int ntrans,
                               const PixelRef *pix, int npix, int ld, double ori_size, cudaStream_t st) {
    if (ntrans <= 0 || npix <= 0) return cudaSuccess;
    dim3 grid((npix + 255) / 256, ntrans);
    k_phase_table<<<grid, 256, 0, st>>>(out, tx, ty, ntrans, pix, npix, ld, ori_size);
    return cudaGetLastError();
}

}  // namespace gbr
