// Device-side setup for topology changes: the energies' preparePrecomputations and the VBD
// per-vertex incidence lists (VBD::computeStencilInfoPerVertex, vbd.cpp:231-268) computed on
// the GPU. Colouring stays on the host (bit-exact greedy order).
//
// The element formulas follow the host classes operation by operation (this file is built
// without FMA contraction, like the host code), so every value except the atan2 of a rest
// bending angle matches the host's to the last bit:
//   discreteBendingEnergy.cpp:48-72, membraneStvkEnergy.cpp:31-71,
//   stableNeoHookeanEnergy.cpp:64-108, stvkEnergy.cpp:69-108, membraneBaraffWitkinEnergy.cpp:42-70,
//   membraneChoiEnergy.cpp:45-70, baraffWitkinBendingEnergy.cpp:55-76,
//   quadraticBendingEnergy.cpp:48-93, springContinuumEnergy.cpp:19-34, staticLoadEnergy.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "api_internal.h"
#include "devbuf.h"
#include "layout.h"

namespace spgx {
namespace {

// Per-stencil failure codes (0 = ok), reported with the reference's messages.
enum PrecomputeError : int {
    kPreOk = 0,
    kPreRestLength,
    kPreRestTheta,
    kPreNotFlat,
    kPreArea,
    kPreVolume,
    kPreQuadTheta,
};

const char *precompute_message(int type, int code)
{
    switch (code) {
    case kPreRestLength: return "Zero/negative rest length invalid";
    case kPreRestTheta: return "Invalid restTheta";
    case kPreNotFlat: return "Rest positions of triangles for membrane energy must have coordinate z=0";
    case kPreArea: return "Rest area of membrane triangle is not positive";
    case kPreVolume: return type == SPGX_ENERGY_STABLE_NEO_HOOKEAN ? "SNH tetrahedron rest volume is not positive"
                                                                   : "tetrahedron rest volume is not positive";
    case kPreQuadTheta: return "Rest theta != 0 not supported for quadratic bending";
    default: return "precomputation failed";
    }
}

struct D3 {
    double x, y, z;
};

__device__ __forceinline__ D3 load3(const double *p, int v) { return {p[3 * size_t(v)], p[3 * size_t(v) + 1], p[3 * size_t(v) + 2]}; }
__device__ __forceinline__ D3 sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 neg(D3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 cross(D3 a, D3 b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double norm(D3 a) { return sqrt(dot(a, a)); }
__device__ __forceinline__ D3 normalized(D3 a)
{
    const double n = norm(a);
    return {a.x / n, a.y / n, a.z / n};
}

// Closed-form inverses and determinant, written as the host's Matrix2/Matrix3 helpers.
__device__ void inverse3(const double *A, double *I)
{
    const double c00 = A[4] * A[8] - A[5] * A[7];
    const double c01 = A[5] * A[6] - A[3] * A[8];
    const double c02 = A[3] * A[7] - A[4] * A[6];
    const double id = 1.0 / (A[0] * c00 + A[1] * c01 + A[2] * c02);
    I[0] = c00 * id;
    I[1] = (A[2] * A[7] - A[1] * A[8]) * id;
    I[2] = (A[1] * A[5] - A[2] * A[4]) * id;
    I[3] = c01 * id;
    I[4] = (A[0] * A[8] - A[2] * A[6]) * id;
    I[5] = (A[2] * A[3] - A[0] * A[5]) * id;
    I[6] = c02 * id;
    I[7] = (A[1] * A[6] - A[0] * A[7]) * id;
    I[8] = (A[0] * A[4] - A[1] * A[3]) * id;
}
__device__ double determinant3(const double *A)
{
    return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) + A[2] * (A[3] * A[7] - A[4] * A[6]);
}
__device__ void inverse2(const double *A, double *I)
{
    const double det = A[0] * A[3] - A[1] * A[2];
    I[0] = A[3] / det;
    I[1] = -A[1] / det;
    I[2] = -A[2] / det;
    I[3] = A[0] / det;
}

// Rest bending angle of a flap (discreteBendingEnergy.cpp:66-70).
__device__ double rest_theta(D3 e0, D3 e3, D3 e4)
{
    const D3 n1 = normalized(cross(e0, e3));
    const D3 n2 = neg(normalized(cross(e0, e4)));
    return atan2(dot(cross(n1, n2), normalized(e0)), dot(n1, n2));
}

// Dm^{-1} and volume of a tet; false when the volume is not positive.
__device__ bool tet_rest(const double *x0, const int *s, double *inv, double &volume)
{
    const D3 p0 = load3(x0, s[0]), p1 = load3(x0, s[1]), p2 = load3(x0, s[2]), p3 = load3(x0, s[3]);
    const D3 c1 = sub(p1, p0), c2 = sub(p2, p0), c3 = sub(p3, p0);
    const double Dm[9] = {c1.x, c2.x, c3.x, c1.y, c2.y, c3.y, c1.z, c2.z, c3.z};
    volume = 1. / 6. * determinant3(Dm);
    if (volume <= 0) return false;
    inverse3(Dm, inv);
    return true;
}

// Dm^{-1} and area of a z = 0 triangle; the error code on failure.
__device__ int tri_rest(const double *x0, const int *s, double *inv, double &area)
{
    const D3 p0 = load3(x0, s[0]), p1 = load3(x0, s[1]), p2 = load3(x0, s[2]);
    if (p0.z != 0.0 || p1.z != 0.0 || p2.z != 0.0) return kPreNotFlat;
    const double u0 = p1.x - p0.x, u1 = p1.y - p0.y;
    const double v0 = p2.x - p0.x, v1 = p2.y - p0.y;
    const double Dm[4] = {u0, v0, u1, v1};
    inverse2(Dm, inv);
    area = (u0 * v1 - v0 * u1) * 0.5;
    return area <= 0 ? kPreArea : kPreOk;
}

__global__ void precompute_kernel(int type, int n, int S, int P, const int *__restrict__ stencils,
                                  const double *__restrict__ x0, const double *__restrict__ material, int mstride,
                                  double *__restrict__ params, int *__restrict__ errors)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int *s = stencils + size_t(i) * S;
    const double *a = material + size_t(i) * mstride;
    double *p = params + size_t(i) * P;
    int err = kPreOk;
    switch (type) {
    case SPGX_ENERGY_SPRING:
    case SPGX_ENERGY_SPRING_CONTINUUM:
    case SPGX_ENERGY_SPRING_SQUARED_CONTINUUM: {
        double L0 = a[0];
        if (L0 <= 0) L0 = norm(sub(load3(x0, s[0]), load3(x0, s[1])));
        if (!(L0 > 0)) {
            err = kPreRestLength;
            break;
        }
        const double k = a[1], c = 1.0 / k;
        p[0] = L0;
        if (type == SPGX_ENERGY_SPRING) {
            p[1] = k;
            p[2] = c;
        } else {
            p[1] = k * L0;
            p[2] = c / L0;
        }
        break;
    }
    case SPGX_ENERGY_SPRING_ANCHOR:
        p[0] = a[0];
        p[1] = a[1];
        p[2] = a[2];
        p[3] = a[3];
        p[4] = 1.0 / a[3];
        break;
    case SPGX_ENERGY_DISCRETE_BENDING:
    case SPGX_ENERGY_BARAFF_WITKIN_BENDING: {
        if (a[0] < -3.12 || a[0] > 3.12) {
            err = kPreRestTheta;
            break;
        }
        const D3 X0 = load3(x0, s[0]), X1 = load3(x0, s[1]);
        const D3 e0 = sub(X1, X0), e3 = sub(load3(x0, s[2]), X1), e4 = sub(load3(x0, s[3]), X1);
        const double k = a[1], c = 1.0 / k;
        p[0] = rest_theta(e0, e3, e4);
        if (type == SPGX_ENERGY_DISCRETE_BENDING) {
            const double f = 2. * 3. * dot(e0, e0) / (0.5 * (norm(cross(e0, e3)) + norm(cross(e0, e4))));
            const double ce = c / f;
            p[1] = 1.0 / ce;
            p[2] = ce;
        } else {
            p[1] = k;
            p[2] = c;
        }
        break;
    }
    case SPGX_ENERGY_MEMBRANE_STVK: {
        double inv[4], area;
        err = tri_rest(x0, s, inv, area);
        if (err) break;
        const double young = a[0], poisson = a[1];
        const double yc = young / (1 - poisson * poisson);
        double C[9] = {yc, yc * poisson, 0, yc * poisson, yc, 0, 0, 0, yc * (1 - poisson) / 2};
        double Ci[9];
        inverse3(C, Ci);
        for (int k = 0; k < 4; ++k) p[k] = inv[k];
        for (int k = 0; k < 9; ++k) {
            p[4 + k] = C[k] * area;
            p[13 + k] = Ci[k] / area;
        }
        break;
    }
    case SPGX_ENERGY_STABLE_NEO_HOOKEAN: {
        double inv[9], volume;
        if (!tet_rest(x0, s, inv, volume)) {
            err = kPreVolume;
            break;
        }
        const double young = a[0], poisson = a[1];
        const double mu = young / (2 * (1 + poisson));
        const double lambda = mu / (1 - 2 * poisson);
        for (int k = 0; k < 9; ++k) p[k] = inv[k];
        p[9] = lambda * volume;
        p[10] = mu * volume;
        p[11] = 1 + mu / lambda;
        p[12] = (1.0 / lambda) / volume;
        p[13] = (1.0 / mu) / volume;
        break;
    }
    case SPGX_ENERGY_STVK:
    case SPGX_ENERGY_STABLE_SQUARED_NEO_HOOKEAN: {
        double inv[9], volume;
        if (!tet_rest(x0, s, inv, volume)) {
            err = kPreVolume;
            break;
        }
        const double young = a[0], poisson = a[1];
        const double mu = young / (2 * (1 + poisson));
        const double lambda = young * poisson / ((1 + poisson) * (1 - 2 * poisson)) + 1e-20;
        for (int k = 0; k < 9; ++k) p[k] = inv[k];
        p[9] = lambda * volume;
        p[10] = mu * volume;
        p[11] = (1.0 / lambda) / volume;
        p[12] = (1.0 / mu) / volume;
        break;
    }
    case SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN:
    case SPGX_ENERGY_MEMBRANE_CHOI: {
        double inv[4], area;
        err = tri_rest(x0, s, inv, area);
        if (err) break;
        const int nk = type == SPGX_ENERGY_MEMBRANE_CHOI ? 4 : 3;
        const double k[4] = {a[0], a[1], a[2], a[2]};
        for (int q = 0; q < 4; ++q) p[q] = inv[q];
        for (int q = 0; q < nk; ++q) {
            p[4 + q] = k[q] * area;
            p[4 + nk + q] = (1.0 / k[q]) / area;
        }
        break;
    }
    case SPGX_ENERGY_QUADRATIC_BENDING: {
        if (a[0] != 0) {
            err = kPreQuadTheta;
            break;
        }
        const D3 X0 = load3(x0, s[0]), X1 = load3(x0, s[1]);
        const D3 e0 = sub(X1, X0), e1 = sub(load3(x0, s[2]), X0), e2 = sub(load3(x0, s[3]), X0);
        const D3 e3 = sub(load3(x0, s[2]), X1), e4 = sub(load3(x0, s[3]), X1);
        auto cot = [](D3 u, D3 v) { return dot(u, v) / norm(cross(u, v)); };
        const double c01 = cot(e0, e1), c02 = cot(e0, e2), c03 = cot(neg(e0), e3), c04 = cot(neg(e0), e4);
        p[0] = c03 + c04;
        p[1] = c01 + c02;
        p[2] = -c01 - c03;
        p[3] = -c02 - c04;
        const double k = a[1] * (3 / (0.5 * (norm(cross(e0, e1)) + norm(cross(e0, e2)))));
        p[4] = k;
        p[5] = 1 / k;
        break;
    }
    case SPGX_ENERGY_STATIC_LOAD: {
        const D3 d = normalized(D3{a[1], a[2], a[3]});
        p[0] = a[0];
        p[1] = d.x;
        p[2] = d.y;
        p[3] = d.z;
        break;
    }
    default: err = -1;
    }
    errors[i] = err;
}

// ---- incidence lists -------------------------------------------------------------------

__global__ void incidence_count_kernel(const int *__restrict__ st, long long n_flat, int ne, int e,
                                       int *__restrict__ counts)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n_flat) atomicAdd(&counts[size_t(st[i]) * ne + e], 1);
}

// Exclusive scan of n ints into 64-bit offsets, one block of 1024 threads walking the array
// in chunks (setup-time work; O(n) with a block-wide scan per chunk).
__global__ void exclusive_scan_kernel(const int *__restrict__ in, long long n, long long *__restrict__ out)
{
    __shared__ long long warp_sums[32];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (long long base = 0; base < n; base += blockDim.x) {
        const long long i = base + threadIdx.x;
        long long v = i < n ? in[i] : 0;
        long long incl = v;
        for (int d = 1; d < 32; d <<= 1) {
            const long long t = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += t;
        }
        if (lane == 31) warp_sums[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            long long w = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
            for (int d = 1; d < 32; d <<= 1) {
                const long long t = __shfl_up_sync(0xffffffffu, w, d);
                if (lane >= d) w += t;
            }
            warp_sums[lane] = w;  // inclusive prefix of warp totals
        }
        __syncthreads();
        const long long before = carry + (warp > 0 ? warp_sums[warp - 1] : 0);
        if (i < n) out[i] = before + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = carry;
}

__global__ void incidence_fill_kernel(const int *__restrict__ st, long long n_flat, int ne, int e,
                                      const long long *__restrict__ off, int *__restrict__ cursor,
                                      long long *__restrict__ keys)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n_flat) return;
    const size_t b = size_t(st[i]) * ne + e;
    const int k = atomicAdd(&cursor[b], 1);
    keys[off[b] + k] = i;
}

// Orders each (vertex, energy) bucket by flat stencil index (the reference's push_back
// order) and writes the (stencil, slot) pairs.
__global__ void incidence_sort_kernel(long long n_buckets, int ne, const int *__restrict__ sizes,
                                      const long long *__restrict__ off, long long *__restrict__ keys,
                                      int *__restrict__ entries)
{
    const long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (b >= n_buckets) return;
    const long long lo = off[b], hi = off[b + 1];
    for (long long j = lo + 1; j < hi; ++j) {
        const long long key = keys[j];
        long long q = j - 1;
        while (q >= lo && keys[q] > key) {
            keys[q + 1] = keys[q];
            --q;
        }
        keys[q + 1] = key;
    }
    const int S = sizes[b % ne];
    for (long long j = lo; j < hi; ++j) {
        entries[2 * j] = static_cast<int>(keys[j] / S);
        entries[2 * j + 1] = static_cast<int>(keys[j] % S);
    }
}

int material_count(int type)
{
    switch (type) {
    case SPGX_ENERGY_SPRING:
    case SPGX_ENERGY_DISCRETE_BENDING:
    case SPGX_ENERGY_MEMBRANE_STVK:
    case SPGX_ENERGY_STABLE_NEO_HOOKEAN:
    case SPGX_ENERGY_STVK:
    case SPGX_ENERGY_STABLE_SQUARED_NEO_HOOKEAN:
    case SPGX_ENERGY_BARAFF_WITKIN_BENDING:
    case SPGX_ENERGY_QUADRATIC_BENDING:
    case SPGX_ENERGY_SPRING_CONTINUUM:
    case SPGX_ENERGY_SPRING_SQUARED_CONTINUUM: return 2;
    case SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN:
    case SPGX_ENERGY_MEMBRANE_CHOI: return 3;
    case SPGX_ENERGY_SPRING_ANCHOR:
    case SPGX_ENERGY_STATIC_LOAD: return 4;
    default: return 0;
    }
}

// One stream and device per call; buffers are released on return.
struct DeviceScope {
    int prev = -1;
    cudaStream_t stream = nullptr;
    spgx_status enter(int device)
    {
        SPGX_CUDA(cudaGetDevice(&prev));
        SPGX_CUDA(cudaSetDevice(device));
        SPGX_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        return SPGX_OK;
    }
    ~DeviceScope()
    {
        if (stream) cudaStreamDestroy(stream);
        if (prev >= 0) cudaSetDevice(prev);
    }
};

}  // namespace
}  // namespace spgx

extern "C" {

int32_t spgx_material_count(int32_t type) { return spgx::material_count(type); }

spgx_status spgx_precompute_params(int32_t type, int32_t n_stencils, const int32_t *stencils, int32_t n_vertices,
                                   const double *x0, const double *material, int32_t material_stride,
                                   double *params, int32_t device)
{
    using namespace spgx;
    SPGX_GUARD_BEGIN
    const int S = stencil_size(type), M = material_count(type), P = spgx_param_count(type);
    if (S == 0 || M == 0) {
        set_error("unsupported energy type " + std::to_string(type));
        return SPGX_ERR_UNSUPPORTED_ENERGY;
    }
    if (n_stencils < 0 || n_vertices < 0 || (n_stencils > 0 && (!stencils || !material || !params)) ||
        (n_vertices > 0 && !x0) || (material_stride != 0 && material_stride < M)) {
        set_error("invalid precompute arguments");
        return SPGX_ERR_INVALID_ARG;
    }
    for (int64_t i = 0; i < int64_t(n_stencils) * S; ++i)
        if (stencils[i] < 0 || stencils[i] >= n_vertices) {
            set_error("stencil contains index to invalid vertex");
            return SPGX_ERR_INVALID_ARG;
        }
    if (n_stencils == 0) return SPGX_OK;
    DeviceScope scope;
    SPGX_TRY_STATUS(scope.enter(device));
    const size_t n = size_t(n_stencils);
    const size_t mrows = material_stride == 0 ? 1 : n;
    DevBuf d_st, d_x0, d_mat, d_par, d_err;
    SPGX_TRY_STATUS(d_st.alloc(n * S * sizeof(int)));
    SPGX_TRY_STATUS(d_x0.alloc(3 * size_t(std::max(1, n_vertices)) * sizeof(double)));
    SPGX_TRY_STATUS(d_mat.alloc(mrows * size_t(material_stride ? material_stride : M) * sizeof(double)));
    SPGX_TRY_STATUS(d_par.alloc(n * P * sizeof(double)));
    SPGX_TRY_STATUS(d_err.alloc(n * sizeof(int)));
    cudaStream_t st = scope.stream;
    SPGX_CUDA(cudaMemcpyAsync(d_st.as<int>(), stencils, n * S * sizeof(int), cudaMemcpyHostToDevice, st));
    SPGX_CUDA(cudaMemcpyAsync(d_x0.as<double>(), x0, 3 * size_t(n_vertices) * sizeof(double), cudaMemcpyHostToDevice, st));
    SPGX_CUDA(cudaMemcpyAsync(d_mat.as<double>(), material,
                              mrows * size_t(material_stride ? material_stride : M) * sizeof(double),
                              cudaMemcpyHostToDevice, st));
    const int threads = 128;
    precompute_kernel<<<unsigned((n + threads - 1) / threads), threads, 0, st>>>(
        type, n_stencils, S, P, d_st.as<int>(), d_x0.as<double>(), d_mat.as<double>(), material_stride,
        d_par.as<double>(), d_err.as<int>());
    SPGX_CUDA(cudaGetLastError());
    std::vector<int> errs(n);
    SPGX_CUDA(cudaMemcpyAsync(params, d_par.as<double>(), n * P * sizeof(double), cudaMemcpyDeviceToHost, st));
    SPGX_CUDA(cudaMemcpyAsync(errs.data(), d_err.as<int>(), n * sizeof(int), cudaMemcpyDeviceToHost, st));
    SPGX_CUDA(cudaStreamSynchronize(st));
    for (size_t i = 0; i < n; ++i)
        if (errs[i] != 0) {
            set_error(std::string(precompute_message(type, errs[i])) + " (stencil " + std::to_string(i) + ")");
            return SPGX_ERR_INVALID_ARG;
        }
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_incidences_device(const spgx_object_desc *obj, int32_t device, int32_t *counts, int32_t *entries,
                                   int64_t *total)
{
    using namespace spgx;
    SPGX_GUARD_BEGIN
    if (!obj || !total || obj->n_vertices < 0 || obj->n_energies < 0 || (obj->n_energies > 0 && !obj->energies)) {
        set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    const int nv = obj->n_vertices, ne = obj->n_energies;
    std::vector<int> sizes(std::max(1, ne), 1);
    long long n_flat_all = 0;
    for (int e = 0; e < ne; ++e) {
        const auto &E = obj->energies[e];
        const int S = stencil_size(E.type);
        if (S == 0) {
            set_error("unsupported energy type " + std::to_string(E.type));
            return SPGX_ERR_UNSUPPORTED_ENERGY;
        }
        if (E.n_stencils < 0 || (E.n_stencils > 0 && !E.stencils)) {
            set_error("invalid energy descriptor");
            return SPGX_ERR_INVALID_ARG;
        }
        for (int64_t i = 0; i < int64_t(E.n_stencils) * S; ++i)
            if (E.stencils[i] < 0 || E.stencils[i] >= nv) {
                set_error("stencil contains index to invalid vertex");
                return SPGX_ERR_INVALID_ARG;
            }
        sizes[e] = S;
        n_flat_all += int64_t(E.n_stencils) * S;
    }
    *total = n_flat_all;
    if (!counts && !entries) return SPGX_OK;
    const long long n_buckets = (long long)nv * ne;
    if (n_buckets == 0) return SPGX_OK;
    DeviceScope scope;
    SPGX_TRY_STATUS(scope.enter(device));
    cudaStream_t st = scope.stream;
    DevBuf d_st, d_cnt, d_off, d_cur, d_keys, d_ent, d_sizes;
    SPGX_TRY_STATUS(d_st.alloc(size_t(std::max<long long>(1, n_flat_all)) * sizeof(int)));
    SPGX_TRY_STATUS(d_cnt.alloc(size_t(n_buckets) * sizeof(int)));
    SPGX_TRY_STATUS(d_cur.alloc(size_t(n_buckets) * sizeof(int)));
    SPGX_TRY_STATUS(d_off.alloc(size_t(n_buckets + 1) * sizeof(long long)));
    SPGX_TRY_STATUS(d_keys.alloc(size_t(std::max<long long>(1, n_flat_all)) * sizeof(long long)));
    SPGX_TRY_STATUS(d_ent.alloc(2 * size_t(std::max<long long>(1, n_flat_all)) * sizeof(int)));
    SPGX_TRY_STATUS(d_sizes.upload(sizes));
    SPGX_CUDA(cudaMemsetAsync(d_cnt.as<int>(), 0, size_t(n_buckets) * sizeof(int), st));
    SPGX_CUDA(cudaMemsetAsync(d_cur.as<int>(), 0, size_t(n_buckets) * sizeof(int), st));
    std::vector<long long> flat_off(ne + 1, 0);
    for (int e = 0; e < ne; ++e) {
        const auto &E = obj->energies[e];
        const long long nf = (long long)E.n_stencils * sizes[e];
        flat_off[e + 1] = flat_off[e] + nf;
        if (nf) SPGX_CUDA(cudaMemcpyAsync(d_st.as<int>() + flat_off[e], E.stencils, size_t(nf) * sizeof(int),
                                          cudaMemcpyHostToDevice, st));
    }
    const int threads = 256;
    for (int e = 0; e < ne; ++e) {
        const long long nf = flat_off[e + 1] - flat_off[e];
        if (nf)
            incidence_count_kernel<<<unsigned((nf + threads - 1) / threads), threads, 0, st>>>(
                d_st.as<int>() + flat_off[e], nf, ne, e, d_cnt.as<int>());
    }
    exclusive_scan_kernel<<<1, 1024, 0, st>>>(d_cnt.as<int>(), n_buckets, d_off.as<long long>());
    // Keys are global flat indices within each energy (the pair's stencil and slot follow).
    for (int e = 0; e < ne; ++e) {
        const long long nf = flat_off[e + 1] - flat_off[e];
        if (nf)
            incidence_fill_kernel<<<unsigned((nf + threads - 1) / threads), threads, 0, st>>>(
                d_st.as<int>() + flat_off[e], nf, ne, e, d_off.as<long long>(), d_cur.as<int>(),
                d_keys.as<long long>());
    }
    incidence_sort_kernel<<<unsigned((n_buckets + threads - 1) / threads), threads, 0, st>>>(
        n_buckets, ne, d_sizes.as<int>(), d_off.as<long long>(), d_keys.as<long long>(), d_ent.as<int>());
    SPGX_CUDA(cudaGetLastError());
    if (counts)
        SPGX_CUDA(cudaMemcpyAsync(counts, d_cnt.as<int>(), size_t(n_buckets) * sizeof(int), cudaMemcpyDeviceToHost, st));
    if (entries && n_flat_all)
        SPGX_CUDA(cudaMemcpyAsync(entries, d_ent.as<int>(), 2 * size_t(n_flat_all) * sizeof(int),
                                  cudaMemcpyDeviceToHost, st));
    SPGX_CUDA(cudaStreamSynchronize(st));
    return SPGX_OK;
    SPGX_GUARD_END
}

}  // extern "C"
