// Launcher for the reference's own GPU path tracer (test and baseline
// infrastructure only; the product never loads it).
//
// The reference renders path-traced frames on the GPU with
// pathTraceOnGPURecursive (src/path_trace.cu:494-555): it copies its median
// kd tree in breadth-first order (KDTreeGPUNode, include/kd_tree_gpu_structs.h,
// built by buildGPUTreeFromKDTree, src/gpu_util.cpp:7-57), the triangles and
// the primary rays to the device, raises the per-thread stack limit to 20 KB,
// and launches evaluatePathKernel (Kajiya) or evaluatePathKernelDiffuse
// (branching mode) over batches of 1,024 pixels, 256 threads per block
// (src/path_trace.cu:525-541). oracle/build_ref.sh compiles
// src/path_trace.cu from the reference's sources into an sm_103a cubin
// (oracle/_ref/prayref_path_trace.cubin); this file loads that cubin with the
// CUDA driver API and repeats the host side of pathTraceOnGPURecursive on
// buffers the caller prepared in the reference's layouts:
//
//   KDTreeGPUNode   88 bytes: int left, int right, bool isLeaf (+7 padding),
//                   size_t firstTriangleIdxIdx, size_t numTriangles,
//                   BoundingBox (6 floats), SplitPlane (uint8 axis + 3
//                   padding, float distance), int ropes[6]
//   Triangle       124 bytes: a, b, c, color (3 floats each), bool
//                   isEmitting (+3 padding), normal, ab, ac, midPoint,
//                   BoundingBox
//   Ray             36 bytes: position, direction, inverse direction
//
// These are the sizes and offsets the reference's headers give on LP64
// hosts (x86-64 and aarch64 alike); the caller checks every index it puts
// into them before the launch.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

#include <cuda.h>

namespace {

thread_local std::string g_err;

int fail(const char *what, CUresult r) {
    const char *name = nullptr;
    cuGetErrorName(r, &name);
    g_err = std::string(what) + ": " + (name ? name : "unknown CUDA error");
    return 1;
}

#define CK(call, what)                         \
    do {                                       \
        CUresult r_ = (call);                  \
        if (r_ != CUDA_SUCCESS) return fail(what, r_); \
    } while (0)

// kernel symbols of src/path_trace.cu:418 and :439 (Itanium C++ ABI)
const char *kKajiya =
    "_ZN4pray18evaluatePathKernelEPNS_13KDTreeGPUNodeEPNS_4cuda8TriangleEPmPNS2_3RayEPNS2_4Vec3EmmmmPh";
const char *kDiffuse =
    "_ZN4pray25evaluatePathKernelDiffuseEPNS_13KDTreeGPUNodeEPNS_4cuda8TriangleEPmPNS2_3RayEPNS2_4Vec3EmmmmPh";

}  // namespace

extern "C" {

const char *refgpu_last_error() { return g_err.c_str(); }

// One frame of the reference's GPU path tracer. nodes: n_nodes x 88 bytes;
// tris: n_tris x 124 bytes; indices: n_idx size_t; rays: n_pixels x 9
// floats; bg: 3 floats. diffuse: 0 = evaluatePathKernel, 1 =
// evaluatePathKernelDiffuse. batch: pixels per launch (the reference uses
// 1,024). frames: how many times the whole frame is rendered (the last one's
// image is returned). image: n_pixels x 3 bytes. ms_out: device time of all
// frames' launches (CUDA events around them). Returns 0, or 1 with
// refgpu_last_error().
int refgpu_path_trace(const char *cubin_path, const void *nodes, uint64_t n_nodes, const void *tris, uint64_t n_tris,
                      const uint64_t *indices, uint64_t n_idx, const float *rays, uint64_t n_pixels, const float *bg,
                      uint64_t max_depth, uint64_t num_samples, int diffuse, uint64_t batch, int frames,
                      uint8_t *image, float *ms_out) {
    if (!cubin_path || !nodes || !tris || !rays || !bg || !image || n_pixels == 0 || batch == 0 || frames < 1) {
        g_err = "invalid argument";
        return 1;
    }
    CK(cuInit(0), "cuInit");
    CUdevice dev;
    CK(cuDeviceGet(&dev, 0), "cuDeviceGet");
    CUcontext ctx;
    CK(cuDevicePrimaryCtxRetain(&ctx, dev), "cuDevicePrimaryCtxRetain");
    CK(cuCtxPushCurrent(ctx), "cuCtxPushCurrent");
    int rc = 0;
    CUmodule mod = nullptr;
    CUdeviceptr d_nodes = 0, d_tris = 0, d_idx = 0, d_rays = 0, d_img = 0, d_bg = 0;
    CUevent e0 = nullptr, e1 = nullptr;
    size_t old_stack = 0;
    bool stack_set = false;
    do {
        CUresult r;
        if ((r = cuModuleLoad(&mod, cubin_path)) != CUDA_SUCCESS) { rc = fail("cuModuleLoad", r); break; }
        CUfunction fn;
        if ((r = cuModuleGetFunction(&fn, mod, diffuse ? kDiffuse : kKajiya)) != CUDA_SUCCESS) {
            rc = fail("cuModuleGetFunction", r);
            break;
        }
        // the reference sets a 20 KB per-thread stack for its recursion
        // (src/path_trace.cu:501-504); restored afterwards
        if ((r = cuCtxGetLimit(&old_stack, CU_LIMIT_STACK_SIZE)) != CUDA_SUCCESS) { rc = fail("cuCtxGetLimit", r); break; }
        if ((r = cuCtxSetLimit(CU_LIMIT_STACK_SIZE, 20 * 1024)) != CUDA_SUCCESS) { rc = fail("cuCtxSetLimit", r); break; }
        stack_set = true;
        const size_t nb = n_nodes * 88, tb = n_tris * 124, ib = (n_idx ? n_idx : 1) * 8, rb = n_pixels * 36;
        if ((r = cuMemAlloc(&d_nodes, nb)) != CUDA_SUCCESS || (r = cuMemAlloc(&d_tris, tb)) != CUDA_SUCCESS ||
            (r = cuMemAlloc(&d_idx, ib)) != CUDA_SUCCESS || (r = cuMemAlloc(&d_rays, rb)) != CUDA_SUCCESS ||
            (r = cuMemAlloc(&d_img, n_pixels * 3)) != CUDA_SUCCESS || (r = cuMemAlloc(&d_bg, 12)) != CUDA_SUCCESS) {
            rc = fail("cuMemAlloc", r);
            break;
        }
        if ((r = cuMemcpyHtoD(d_nodes, nodes, nb)) != CUDA_SUCCESS || (r = cuMemcpyHtoD(d_tris, tris, tb)) != CUDA_SUCCESS ||
            (n_idx && (r = cuMemcpyHtoD(d_idx, indices, n_idx * 8)) != CUDA_SUCCESS) ||
            (r = cuMemcpyHtoD(d_rays, rays, rb)) != CUDA_SUCCESS || (r = cuMemcpyHtoD(d_bg, bg, 12)) != CUDA_SUCCESS) {
            rc = fail("cuMemcpyHtoD", r);
            break;
        }
        if ((r = cuEventCreate(&e0, CU_EVENT_DEFAULT)) != CUDA_SUCCESS || (r = cuEventCreate(&e1, CU_EVENT_DEFAULT)) != CUDA_SUCCESS) {
            rc = fail("cuEventCreate", r);
            break;
        }
        const unsigned block = 256;
        if ((r = cuEventRecord(e0, 0)) != CUDA_SUCCESS) { rc = fail("cuEventRecord", r); break; }
        for (int f = 0; f < frames && rc == 0; f++) {
            for (uint64_t start = 0; start < n_pixels; start += batch) {
                uint64_t end = start + batch < n_pixels ? start + batch : n_pixels;
                // getNeededGridDimension (src/path_trace.cu:459-471): x up to 65,535, then y
                const uint64_t blocks = (end - start + block - 1) / block;
                const unsigned gx = blocks > 65535 ? 65535u : (unsigned)blocks;
                const unsigned gy = blocks > 65535 ? (unsigned)((blocks + 65534) / 65535) : 1u;
                uint64_t md = max_depth, ns = num_samples, s0 = start, s1 = end;
                void *args[] = {&d_nodes, &d_tris, &d_idx, &d_rays, &d_bg, &md, &ns, &s0, &s1, &d_img};
                if ((r = cuLaunchKernel(fn, gx, gy, 1, block, 1, 1, 0, 0, args, nullptr)) != CUDA_SUCCESS) {
                    rc = fail("cuLaunchKernel", r);
                    break;
                }
            }
        }
        if (rc) break;
        if ((r = cuEventRecord(e1, 0)) != CUDA_SUCCESS) { rc = fail("cuEventRecord", r); break; }
        if ((r = cuEventSynchronize(e1)) != CUDA_SUCCESS) { rc = fail("kernel execution", r); break; }
        float ms = 0.f;
        if ((r = cuEventElapsedTime(&ms, e0, e1)) != CUDA_SUCCESS) { rc = fail("cuEventElapsedTime", r); break; }
        if (ms_out) *ms_out = ms;
        if ((r = cuMemcpyDtoH(image, d_img, n_pixels * 3)) != CUDA_SUCCESS) { rc = fail("cuMemcpyDtoH", r); break; }
    } while (false);
    if (e0) cuEventDestroy(e0);
    if (e1) cuEventDestroy(e1);
    for (CUdeviceptr p : {d_nodes, d_tris, d_idx, d_rays, d_img, d_bg})
        if (p) cuMemFree(p);
    if (stack_set) cuCtxSetLimit(CU_LIMIT_STACK_SIZE, old_stack);
    if (mod) cuModuleUnload(mod);
    cuCtxPopCurrent(nullptr);
    cuDevicePrimaryCtxRelease(dev);
    return rc;
}

}  // extern "C"
