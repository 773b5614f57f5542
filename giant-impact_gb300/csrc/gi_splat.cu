// gi_splat.cu -- headless point splat of a frame into an RGB image.
//
// The reference draws each element as a 2-pixel GL point coloured by
// origin and material (drawPictureNormal, impactBasicFunctions.h:666-697;
// colours commonSetup.h:125-128) through gluLookAt + glFrustum
// (impactAddTime.cu:535-538).  Here the same camera model is evaluated in
// CUDA without any graphics API:
//   eye space   x_e = s.(p - eye), y_e = u.(p - eye), depth = f.(p - eye)
//               with f = (center - eye)/|..|, s = f x up/|..|, u = s x f;
//   projection  x_ndc = (near / half) x_e / depth (glFrustum(-half, half,
//               -half, half, near, far)), visible for near <= depth <= far;
//   raster      a point_size x point_size square of pixels around the
//               window position, top row first.
// Every covered pixel takes atomicMin of (depth bits << 32 | rgb): the
// nearest element wins and equal depths resolve to the smaller colour, so
// the image does not depend on launch order.  All arithmetic is FP32 with
// explicit roundings (no contraction), so a CPU restatement can reproduce
// the image exactly.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gi_internal.h"

namespace gi {

struct SplatCam {
    float eye[3], s[3], u[3], f[3];
    float k;           // near / half
    float near_plane, far_plane;
    float half_w, half_h;  // width / 2, height / 2
    int width, height, point_size;
    unsigned int rgb[6];   // Fe body 1, Fe body 2, Si body 1, Si body 2, Earth, Moon
    int b0, b1, b2;
};

__device__ __forceinline__ float dot_rn(const float a[3], float x, float y, float z)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(a[0], x), __fmul_rn(a[1], y)), __fmul_rn(a[2], z));
}

// scope == nullptr: every element, coloured by origin and material.
// Otherwise the analysis picture: only elements of scope 1 (Earth, blue)
// and 2 (Moon, white).
__global__ void __launch_bounds__(256)
splat_kernel(const float4 *__restrict__ pos, int n, const unsigned char *__restrict__ scope,
             const __grid_constant__ SplatCam cam, unsigned long long *__restrict__ zbuf)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int c;
        if (scope) {
            const int sc = scope[i];
            if (sc != 1 && sc != 2) continue;
            c = 3 + sc;
        } else {
            c = i < cam.b0 ? 0 : (i < cam.b1 ? 1 : (i < cam.b2 ? 2 : 3));
        }
        const float4 p = pos[i];
        const float dx = __fsub_rn(p.x, cam.eye[0]), dy = __fsub_rn(p.y, cam.eye[1]),
                    dz = __fsub_rn(p.z, cam.eye[2]);
        const float depth = dot_rn(cam.f, dx, dy, dz);
        if (!(depth >= cam.near_plane && depth <= cam.far_plane)) continue;
        const float xe = dot_rn(cam.s, dx, dy, dz), ye = dot_rn(cam.u, dx, dy, dz);
        const float xn = __fdiv_rn(__fmul_rn(cam.k, xe), depth);
        const float yn = __fdiv_rn(__fmul_rn(cam.k, ye), depth);
        if (!(fabsf(xn) <= 2.0f && fabsf(yn) <= 2.0f)) continue;
        const float wx = __fmul_rn(__fadd_rn(xn, 1.0f), cam.half_w);
        const float wy = __fmul_rn(__fsub_rn(1.0f, yn), cam.half_h);
        const float lo = 0.5f * (float)cam.point_size - 0.5f;
        const int x0 = (int)floorf(__fsub_rn(wx, lo)), y0 = (int)floorf(__fsub_rn(wy, lo));
        const unsigned long long key =
            ((unsigned long long)__float_as_uint(depth) << 32) | cam.rgb[c];
        for (int yy = y0; yy < y0 + cam.point_size; ++yy) {
            if (yy < 0 || yy >= cam.height) continue;
            for (int xx = x0; xx < x0 + cam.point_size; ++xx) {
                if (xx < 0 || xx >= cam.width) continue;
                atomicMin(&zbuf[(size_t)yy * cam.width + xx], key);
            }
        }
    }
}

__global__ void __launch_bounds__(256)
resolve_kernel(const unsigned long long *__restrict__ zbuf, size_t npix,
               unsigned char *__restrict__ rgb)
{
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < npix;
         k += (size_t)gridDim.x * blockDim.x) {
        const unsigned long long z = zbuf[k];
        const unsigned int c = z == ~0ull ? 0u : (unsigned int)(z & 0xffffffu);
        rgb[3 * k + 0] = (unsigned char)(c >> 16);
        rgb[3 * k + 1] = (unsigned char)(c >> 8);
        rgb[3 * k + 2] = (unsigned char)c;
    }
}

}  // namespace gi

namespace {

int cuda_status(cudaError_t e, const char *what)
{
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    return gi_internal_fail(e == cudaErrorMemoryAllocation ? GI_ERR_OUT_OF_MEMORY : GI_ERR_CUDA, buf);
}

unsigned int pack_rgb(double r, double g, double b)
{
    auto q = [](double c) { return (unsigned int)std::lround(std::min(1.0, std::max(0.0, c)) * 255.0); };
    return (q(r) << 16) | (q(g) << 8) | q(b);
}

}  // namespace

extern "C" int gi_view_basis(const gi_view *v, float out[12])
{
    if (!v || !out) return gi_internal_fail(GI_ERR_INVALID_ARG, "gi_view_basis: NULL argument");
    double f[3], s[3], u[3];
    for (int k = 0; k < 3; ++k) f[k] = (double)v->center[k] - v->eye[k];
    double fm = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    if (!(fm > 0.0)) return gi_internal_fail(GI_ERR_PARAMS, "gi_view: eye == center");
    for (double &x : f) x /= fm;
    s[0] = f[1] * v->up[2] - f[2] * v->up[1];
    s[1] = f[2] * v->up[0] - f[0] * v->up[2];
    s[2] = f[0] * v->up[1] - f[1] * v->up[0];
    double sm = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    if (!(sm > 0.0)) return gi_internal_fail(GI_ERR_PARAMS, "gi_view: up is parallel to the view");
    for (double &x : s) x /= sm;
    u[0] = s[1] * f[2] - s[2] * f[1];
    u[1] = s[2] * f[0] - s[0] * f[2];
    u[2] = s[0] * f[1] - s[1] * f[0];
    for (int k = 0; k < 3; ++k) {
        out[k] = (float)s[k];
        out[3 + k] = (float)u[k];
        out[6 + k] = (float)f[k];
        out[9 + k] = v->eye[k];
    }
    return GI_OK;
}

namespace {

// gi_splat (bounds, scope == nullptr) and gi_splat_scope (scope, bounds == nullptr).
int splat_impl(gi_ctx *ctx, const float *pos, int n, const int *bounds,
               const unsigned char *scope, const gi_view *view, unsigned char *rgb, void *stream)
{
    if (!ctx || (!bounds && !scope) || !view || !rgb || n < 0 || (n > 0 && !pos))
        return gi_internal_fail(GI_ERR_INVALID_ARG, "gi_splat: NULL argument or n < 0");
    if (view->width <= 0 || view->height <= 0 || view->width > 16384 || view->height > 16384 ||
        view->point_size < 1 || view->point_size > 64)
        return gi_internal_fail(GI_ERR_INVALID_ARG, "gi_splat: image 1..16384 px, point 1..64 px");
    if (!(view->frustum_half > 0.0f) || !(view->near_plane > 0.0f) ||
        !(view->far_plane > view->near_plane))
        return gi_internal_fail(GI_ERR_INVALID_ARG, "gi_splat: frustum needs half > 0, 0 < near < far");
    if (reinterpret_cast<uintptr_t>(pos) % 16)
        return gi_internal_fail(GI_ERR_ALIGNMENT, "gi_splat: pos not 16-byte aligned");
    float basis[12];
    if (int st = gi_view_basis(view, basis)) return st;
    gi::SplatCam cam;
    for (int k = 0; k < 3; ++k) {
        cam.s[k] = basis[k];
        cam.u[k] = basis[3 + k];
        cam.f[k] = basis[6 + k];
        cam.eye[k] = basis[9 + k];
    }
    cam.k = view->near_plane / view->frustum_half;
    cam.near_plane = view->near_plane;
    cam.far_plane = view->far_plane;
    cam.half_w = 0.5f * (float)view->width;
    cam.half_h = 0.5f * (float)view->height;
    cam.width = view->width;
    cam.height = view->height;
    cam.point_size = view->point_size;
    cam.rgb[0] = pack_rgb(1.0, 1.0, 0.0);     // ColorBody1Core
    cam.rgb[1] = pack_rgb(1.0, 0.0, 0.0);     // ColorBody2Core
    cam.rgb[2] = pack_rgb(0.39, 0.26, 0.13);  // ColorBody1Mantle
    cam.rgb[3] = pack_rgb(0.71, 0.40, 0.11);  // ColorBody2Mantle
    cam.rgb[4] = pack_rgb(0.0, 0.0, 1.0);     // Earth (drawAnalysisPicture)
    cam.rgb[5] = pack_rgb(1.0, 1.0, 1.0);     // Moon
    cam.b0 = bounds ? bounds[0] : 0;
    cam.b1 = bounds ? bounds[1] : 0;
    cam.b2 = bounds ? bounds[2] : 0;
    const int dev = gi_internal_ctx_device(ctx);
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
    struct Restore {
        int prev, dev;
        ~Restore()
        {
            if (prev != dev && prev >= 0) cudaSetDevice(prev);
        }
    } restore{prev, dev};
    cudaStream_t s = (cudaStream_t)stream;
    const size_t npix = (size_t)view->width * view->height;
    unsigned char *buf = nullptr;
    cudaError_t e = cudaMallocAsync(&buf, npix * 8 + npix * 3, s);
    if (e != cudaSuccess) return cuda_status(e, "cudaMallocAsync");
    unsigned long long *zbuf = reinterpret_cast<unsigned long long *>(buf);
    unsigned char *img = buf + npix * 8;
    do {
        if ((e = cudaMemsetAsync(zbuf, 0xff, npix * 8, s)) != cudaSuccess) break;
        if (n > 0)
            gi::splat_kernel<<<std::min((n + 255) / 256, 8192), 256, 0, s>>>(
                reinterpret_cast<const float4 *>(pos), n, scope, cam, zbuf);
        gi::resolve_kernel<<<(int)std::min<size_t>((npix + 255) / 256, 8192), 256, 0, s>>>(zbuf, npix,
                                                                                          img);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(rgb, img, npix * 3, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
    } while (false);
    const cudaError_t ef = cudaFreeAsync(buf, s);
    if (e == cudaSuccess) e = ef;
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_status(e, "gi_splat");
    return GI_OK;
}

}  // namespace

extern "C" int gi_splat(gi_ctx *ctx, const float *pos, int n, const int bounds[3],
                        const gi_view *view, unsigned char *rgb, void *stream)
{
    if (!bounds) return gi_internal_fail(GI_ERR_INVALID_ARG, "gi_splat: bounds is NULL");
    return splat_impl(ctx, pos, n, bounds, nullptr, view, rgb, stream);
}

extern "C" int gi_splat_scope(gi_ctx *ctx, const float *pos, int n, const unsigned char *scope,
                              const gi_view *view, unsigned char *rgb, void *stream)
{
    if (!scope) return gi_internal_fail(GI_ERR_INVALID_ARG, "gi_splat_scope: scope is NULL");
    return splat_impl(ctx, pos, n, nullptr, scope, view, rgb, stream);
}

extern "C" int gi_write_ppm(const char *path, const unsigned char *rgb, int width, int height)
{
    if (!path || !rgb || width <= 0 || height <= 0)
        return gi_internal_fail(GI_ERR_INVALID_ARG, "gi_write_ppm: bad argument");
    FILE *f = std::fopen(path, "wb");
    if (!f) return gi_internal_fail(GI_ERR_IO, "gi_write_ppm: cannot open the file");
    std::fprintf(f, "P6\n%d %d\n255\n", width, height);
    const size_t bytes = (size_t)width * height * 3;
    const bool ok = std::fwrite(rgb, 1, bytes, f) == bytes;
    if (std::fclose(f) != 0 || !ok) return gi_internal_fail(GI_ERR_IO, "gi_write_ppm: write failed");
    return GI_OK;
}

extern "C" int gi_render_frames(int device, const char *info_dir, const char *frames_path,
                                const gi_view *view, int every, const char *out_prefix,
                                long long *written)
{
    if (!info_dir || !frames_path || !view || !out_prefix || every < 1)
        return gi_internal_fail(GI_ERR_INVALID_ARG, "gi_render_frames: bad argument");
    gi_body_params b;
    std::string path = std::string(info_dir) + "/targetImpactorParameters";
    if (int st = gi_read_body_params(path.c_str(), &b))
        return gi_internal_fail(st, (path + ": cannot read").c_str());
    const int n = b.n;
    const int bounds[3] = {b.nfe1, b.nfe1 + b.nfe2, b.nfe1 + b.nfe2 + b.nsi1};
    long long count = 0;
    if (int st = gi_frames_count(frames_path, n, &count))
        return gi_internal_fail(st, "gi_render_frames: frame file unreadable or truncated");
    gi_ctx *ctx = nullptr;
    if (int st = gi_ctx_create(&ctx, device)) return st;
    std::vector<float> pos(4 * (size_t)n), vel(4 * (size_t)n);
    std::vector<unsigned char> rgb((size_t)view->width * view->height * 3);
    float *dpos = nullptr;
    int st = GI_OK;
    if (cudaSetDevice(device) != cudaSuccess || cudaMalloc(&dpos, (size_t)(n > 0 ? n : 1) * 16) != cudaSuccess)
        st = gi_internal_fail(GI_ERR_OUT_OF_MEMORY, "gi_render_frames: device buffer");
    long long done = 0;
    for (long long fr = 0; st == GI_OK && fr < count; fr += every) {
        float t = 0.0f;
        if ((st = gi_frames_read(frames_path, n, fr, &t, pos.data(), vel.data()))) break;
        if (cudaMemcpy(dpos, pos.data(), (size_t)n * 16, cudaMemcpyHostToDevice) != cudaSuccess) {
            st = gi_internal_fail(GI_ERR_CUDA, "gi_render_frames: upload");
            break;
        }
        if ((st = gi_splat(ctx, dpos, n, bounds, view, rgb.data(), nullptr))) break;
        char name[64];
        std::snprintf(name, sizeof name, "%05lld.ppm", fr);
        if ((st = gi_write_ppm((std::string(out_prefix) + name).c_str(), rgb.data(), view->width,
                               view->height)))
            break;
        ++done;
    }
    cudaFree(dpos);
    gi_ctx_destroy(ctx);
    if (written) *written = done;
    return st;
}
