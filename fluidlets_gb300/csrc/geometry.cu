// geometry.cu -- the reference's sphere discretizations and the mean
// nearest-neighbour spacing, generated on the device (request set-up without a
// host round trip).  Same arithmetic, in the same order, as the reference's
// NumPy code (geometry/spheres.py); the _rn intrinsics keep the compiler from
// fusing a multiply and an add that NumPy rounds separately.
#include <algorithm>

#include "flg_common.cuh"

namespace flg {

// geometry/spheres.py:7-13: k = i + 1/2, phi = arccos(1 - 2k/n), theta = pi (1 + sqrt 5) k
__global__ void fibonacci_kernel(int64_t n, double radius, double cx, double cy, double cz, double *out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double k = (double)i + 0.5;
    const double phi = acos(__dsub_rn(1.0, __ddiv_rn(__dmul_rn(2.0, k), (double)n)));
    const double theta = __dmul_rn(__dmul_rn(3.141592653589793, __dadd_rn(1.0, sqrt(5.0))), k);
    const double sp = sin(phi);
    out[3 * i] = __dadd_rn(__dmul_rn(radius, __dmul_rn(cos(theta), sp)), cx);
    out[3 * i + 1] = __dadd_rn(__dmul_rn(radius, __dmul_rn(sin(theta), sp)), cy);
    out[3 * i + 2] = __dadd_rn(__dmul_rn(radius, cos(phi)), cz);
}

// geometry/spheres.py:33-52: face f = 2 axis + (sign > 0), point (a, b) of the cell-centred
// n x n grid s = linspace(-1 + 1/n, 1 - 1/n, n), projected radially
__global__ void cube_sphere_kernel(int64_t n, double radius, double cx, double cy, double cz, double *out) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= 6 * n * n) return;
    const int64_t f = p / (n * n), ab = p % (n * n), ia = ab / n, ib = ab % n;
    const double start = __dadd_rn(-1.0, __ddiv_rn(1.0, (double)n)), stop = __dsub_rn(1.0, __ddiv_rn(1.0, (double)n));
    // np.linspace: i * step + start, step = (stop - start) / (n - 1), the last point exactly stop
    auto lin = [&](int64_t i) {
        if (n > 1 && i == n - 1) return stop;
        if (n == 1) return start;
        const double step = __ddiv_rn(__dsub_rn(stop, start), (double)(n - 1));
        return __dadd_rn(__dmul_rn((double)i, step), start);
    };
    const double A = lin(ia), B = lin(ib), sgn = (f & 1) ? 1.0 : -1.0;
    const int axis = (int)(f >> 1);
    double v[3];
    v[axis] = sgn;
    v[axis == 0 ? 1 : 0] = A;
    v[axis == 2 ? 1 : 2] = B;
    const double nrm = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])), __dmul_rn(v[2], v[2])));
    const double c[3] = {cx, cy, cz};
#pragma unroll
    for (int d = 0; d < 3; d++) out[3 * p + d] = __dadd_rn(__dmul_rn(radius, __ddiv_rn(v[d], nrm)), c[d]);
}

// distance from each point to its nearest other point (exhaustive, FP64)
__global__ void __launch_bounds__(256) nn_distance_kernel(const double *pts, int64_t n, double *dist) {
    __shared__ double fx[1024], fy[1024], fz[1024];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double px = 0.0, py = 0.0, pz = 0.0;
    if (i < n) px = pts[3 * i], py = pts[3 * i + 1], pz = pts[3 * i + 2];
    double best = INFINITY;
    for (int64_t t0 = 0; t0 < n; t0 += 1024) {
        const int nt = (int)min((int64_t)1024, n - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < nt; k += blockDim.x) {
            fx[k] = pts[3 * (t0 + k)];
            fy[k] = pts[3 * (t0 + k) + 1];
            fz[k] = pts[3 * (t0 + k) + 2];
        }
        __syncthreads();
        for (int k = 0; k < nt; k++) {
            if (t0 + k == i) continue;
            const double dx = px - fx[k], dy = py - fy[k], dz = pz - fz[k];
            best = fmin(best, dx * dx + dy * dy + dz * dz);
        }
    }
    if (i < n) dist[i] = sqrt(best);
}

// mean of dist[0..n) in a fixed order (one CTA, per-thread partial sums in index order)
__global__ void __launch_bounds__(256) mean_kernel(const double *dist, int64_t n, double *mean) {
    __shared__ double part[256];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += dist[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *mean = part[0] / (double)n;
}

}  // namespace flg

using namespace flg;

extern "C" int flg_fibonacci_sphere(int64_t n, double radius, const double *center, double *out, void *stream) {
    FLG_REQUIRE(n >= 0 && center, "bad sphere arguments");
    if (n == 0) return FLG_OK;
    FLG_REQUIRE(out, "null pointer");
    fibonacci_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, as_stream(stream)>>>(n, radius, center[0], center[1],
                                                                                center[2], out);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}

extern "C" int flg_cube_sphere(int64_t n, double radius, const double *center, double *out, void *stream) {
    FLG_REQUIRE(n >= 0 && center, "bad sphere arguments");
    if (n == 0) return FLG_OK;
    FLG_REQUIRE(out, "null pointer");
    cube_sphere_kernel<<<(unsigned)ceil_div(6 * n * n, 256), 256, 0, as_stream(stream)>>>(n, radius, center[0],
                                                                                          center[1], center[2], out);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}

extern "C" int flg_mean_nn_spacing(const double *points, int64_t n, double *mean, void *work, size_t work_bytes,
                                   void *stream) {
    FLG_REQUIRE(n >= 2, "the nearest-neighbour spacing needs at least two points");
    FLG_REQUIRE(points && mean, "null pointer");
    Arena ar(work, work_bytes);
    double *dist = ar.take<double>(n);
    FLG_REQUIRE(dist, "workspace too small (%zu bytes)", work_bytes);
    cudaStream_t st = as_stream(stream);
    nn_distance_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(points, n, dist);
    FLG_LAUNCH_CHECK();
    mean_kernel<<<1, 256, 0, st>>>(dist, n, mean);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}

extern "C" size_t flg_mean_nn_spacing_workspace(int64_t n) {
    CountingArena c;
    c.take<double>(std::max<int64_t>(n, 1));
    return c.bytes();
}
