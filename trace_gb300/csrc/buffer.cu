// Render targets of pkg/pt/buffer.go kept on the device.
//
//   PixelBuffer (buffer.go:14-58)  every pixel is the running mean of all the
//                                  samples added to it, across RenderToBuffer
//                                  calls (Pixel.addSample, buffer.go:19-26)
//   FrameBuffer (buffer.go:71-116) every pixel holds the last sample written
//                                  (addSample overwrites, buffer.go:91-93)
//   ToImage (buffer.go:60-69, 104-116 with Color.goColor, math.go:20-25)
//                                  gamma 2 (square root), clamp to [0, 1],
//                                  x255 truncated to a byte, alpha 255, written
//                                  at row height - (i / width): buffer row 0
//                                  falls outside the image and image row 0
//                                  stays (0, 0, 0, 0)
//
// RenderToBuffer passes its spp samples over every pixel (render.go:117-124).
// Into a PixelBuffer the call's spp-sample mean is blended into the running
// mean with weight spp / (samples so far + spp).  A FrameBuffer keeps only
// the sample of the call's last pass, which overwrote the earlier ones, so
// only that pass is traced.  The reference seeds every call from the clock;
// here call k on a buffer draws with seed + k * 0x9E3779B97F4A7C15, so that
// successive calls add new samples and the first call equals gbt_render's
// image for the same parameters.
#include <cuda_runtime.h>

#include <cmath>

#include "gbt_internal.cuh"

struct gbt_buffer {
    gbt_ctx *ctx = nullptr;
    int32_t kind = GBT_BUFFER_PIXEL;
    int32_t width = 0, height = 0;
    uint64_t samples = 0;  // samples per pixel added so far (PixelBuffer), 0 or 1 (FrameBuffer)
    uint64_t calls = 0;    // RenderToBuffer calls so far
    float *d_rgb = nullptr;   // width*height*3, row y = 0 first (buffer.go:47-49)
    float *d_call = nullptr;  // this call's image before it is blended in (PixelBuffer)
    uint8_t *d_rgba = nullptr;  // ToImage staging, width*height*4
};

namespace {

// m <- m + (c - m) * w, the running mean of buffer.go:23-25 taken over a whole call
__global__ void k_blend(float *__restrict__ mean, const float *__restrict__ call, uint32_t n, float w) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const float m = mean[i];
        mean[i] = m + (call[i] - m) * w;
    }
}

// Color.goColor (math.go:20-25) of one channel: sqrt in float64, Clamp (util.go:32-40),
// x255 and Go's float64 -> uint8 truncation.  NaN (sqrt of a negative, which Clamp passes
// through) converts to 0 as on amd64 and arm64.
__device__ __forceinline__ uint8_t go_channel(float c) {
    double s = sqrt((double)c);
    if (s != s) return 0;
    if (s < 0.0) s = 0.0;
    if (s > 1.0) s = 1.0;
    return (uint8_t)(int)(s * 255.0);
}

__global__ void k_to_image(const float *__restrict__ rgb, uint8_t *__restrict__ rgba, uint32_t w, uint32_t h) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;  // image pixel
    if (i >= w * h) return;
    const uint32_t x = i % w, y = i / w;
    uchar4 px = make_uchar4(0, 0, 0, 0);  // image row 0 is never set (buffer.go:65)
    if (y > 0) {
        const uint32_t src = (h - y) * w + x;  // buffer row h - y lands on image row y
        px = make_uchar4(go_channel(rgb[3 * (size_t)src]), go_channel(rgb[3 * (size_t)src + 1]),
                         go_channel(rgb[3 * (size_t)src + 2]), 255);
    }
    reinterpret_cast<uchar4 *>(rgba)[i] = px;
}

}  // namespace

extern "C" int gbt_buffer_create(gbt_ctx *ctx, int32_t kind, int32_t width, int32_t height, gbt_buffer **out) {
    if (!ctx || !out) return GBT_EINVAL;
    *out = nullptr;
    if (kind != GBT_BUFFER_PIXEL && kind != GBT_BUFFER_FRAME)
        return gbt_fail(ctx, GBT_EINVAL, "buffer_create: kind must be GBT_BUFFER_PIXEL or GBT_BUFFER_FRAME");
    if (width < 2 || height < 2 || (uint64_t)width * (uint64_t)height >= (1ull << 31))
        return gbt_fail(ctx, GBT_EINVAL, "buffer_create: width, height >= 2 and width*height < 2^31");
    gbt_buffer *b = new gbt_buffer;
    b->ctx = ctx;
    b->kind = kind;
    b->width = width;
    b->height = height;
    const size_t npix = (size_t)width * height;
    cudaError_t e = cudaMalloc(&b->d_rgb, npix * 3 * sizeof(float));
    if (e == cudaSuccess && kind == GBT_BUFFER_PIXEL) e = cudaMalloc(&b->d_call, npix * 3 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_rgba, npix * 4);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_rgb, 0, npix * 3 * sizeof(float), ctx->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaFree(b->d_rgb);
        cudaFree(b->d_call);
        cudaFree(b->d_rgba);
        delete b;
        return gbt_fail(ctx, GBT_ENOMEM, "buffer_create: device allocation");
    }
    *out = b;
    return GBT_OK;
}

extern "C" int gbt_buffer_destroy(gbt_buffer *b) {
    if (!b) return GBT_EINVAL;
    cudaStreamSynchronize(b->ctx->stream);
    cudaFree(b->d_rgb);
    cudaFree(b->d_call);
    cudaFree(b->d_rgba);
    delete b;
    return GBT_OK;
}

// Adds an image of `spp` samples per pixel (already averaged) to the buffer.
static int buffer_add(gbt_ctx *ctx, gbt_buffer *b, const float *d_img, uint64_t spp) {
    const uint32_t n = (uint32_t)((size_t)b->width * b->height * 3);
    if (b->kind == GBT_BUFFER_FRAME || b->samples == 0) {
        if (d_img != b->d_rgb)
            GBT_CUDA(ctx, cudaMemcpyAsync(b->d_rgb, d_img, (size_t)n * sizeof(float), cudaMemcpyDeviceToDevice,
                                          ctx->stream));
        b->samples = b->kind == GBT_BUFFER_FRAME ? 1 : spp;
    } else {
        const double w = (double)spp / (double)(b->samples + spp);
        k_blend<<<(n + 255) / 256, 256, 0, ctx->stream>>>(b->d_rgb, d_img, n, (float)w);
        GBT_CUDA(ctx, cudaGetLastError());
        ctx->last_stats.kernel_launches += 1;
        b->samples += spp;
    }
    return GBT_OK;
}

extern "C" int gbt_buffer_add_async(gbt_ctx *ctx, gbt_buffer *b, const float *d_rgb, int32_t samples) {
    if (!ctx || !b || !d_rgb || b->ctx != ctx || samples < 1) return GBT_EINVAL;
    return buffer_add(ctx, b, d_rgb, (uint64_t)samples);
}

extern "C" int gbt_render_to_buffer_async(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam,
                                          const gbt_render_params *p, gbt_buffer *b) {
    if (!ctx || !bvh || !cam || !p || !b || b->ctx != ctx) return GBT_EINVAL;
    if (p->width != b->width || p->height != b->height)
        return gbt_fail(ctx, GBT_EINVAL, "render_to_buffer: params width/height differ from the buffer's");
    if (p->spp < 1) return gbt_fail(ctx, GBT_EINVAL, "render_to_buffer: spp >= 1");
    gbt_render_params q = *p;
    q.seed = p->seed + b->calls * 0x9E3779B97F4A7C15ull;
    // a FrameBuffer keeps the sample of the last pass, which overwrote the earlier ones
    if (b->kind == GBT_BUFFER_FRAME) q.spp = 1;
    // the first image into a buffer (and every FrameBuffer image) is written in place
    const bool direct = b->kind == GBT_BUFFER_FRAME || b->samples == 0;
    float *dst = direct ? b->d_rgb : b->d_call;
    int rc = gbt_render_enqueue(ctx, bvh, cam, &q, dst);
    if (rc) return rc;
    rc = buffer_add(ctx, b, dst, (uint64_t)q.spp);
    if (rc) return rc;
    b->calls++;
    return GBT_OK;
}

extern "C" int gbt_render_to_buffer(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, const gbt_render_params *p,
                                    gbt_buffer *b, gbt_render_stats *stats) {
    int rc = gbt_render_to_buffer_async(ctx, bvh, cam, p, b);
    if (rc) return rc;
    rc = gbt_check_device_error(ctx, "render_to_buffer");
    if (rc) return rc;
    GBT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (stats) return gbt_render_last_stats(ctx, stats);
    return GBT_OK;
}

extern "C" int gbt_buffer_read(gbt_ctx *ctx, gbt_buffer *b, float *rgb, uint64_t *samples) {
    if (!ctx || !b || b->ctx != ctx) return GBT_EINVAL;
    if (samples) *samples = b->samples;
    if (rgb) {
        GBT_CUDA(ctx, cudaMemcpyAsync(rgb, b->d_rgb, (size_t)b->width * b->height * 3 * sizeof(float),
                                      cudaMemcpyDeviceToHost, ctx->stream));
        GBT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return GBT_OK;
}

extern "C" int gbt_buffer_to_image(gbt_ctx *ctx, gbt_buffer *b, uint8_t *rgba) {
    if (!ctx || !b || !rgba || b->ctx != ctx) return GBT_EINVAL;
    const uint32_t npix = (uint32_t)((size_t)b->width * b->height);
    k_to_image<<<(npix + 255) / 256, 256, 0, ctx->stream>>>(b->d_rgb, b->d_rgba, (uint32_t)b->width,
                                                            (uint32_t)b->height);
    GBT_CUDA(ctx, cudaGetLastError());
    GBT_CUDA(ctx, cudaMemcpyAsync(rgba, b->d_rgba, (size_t)npix * 4, cudaMemcpyDeviceToHost, ctx->stream));
    GBT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GBT_OK;
}
