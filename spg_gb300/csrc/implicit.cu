// GB300 implicit Euler (one Newton step per substep), the GPU counterpart of
// spg::solver::ImplicitEulerNewtonDx::step (spg/source/sim/solver/implicitEulerNewtonDx.cpp:11-65)
// with the system assembly and linear solve of ImplicitEulerBase
// (spg/source/sim/solver/implicitEulerBase.cpp:102-240):
//
//   per substep: x0 = x; y = x + h v (integrateVelocities, particleGroup.cpp:57-63);
//   f = M g - grad E(y) (getSystemForce); K = -hess E(y) (getSystemStiffnessMatrix, full element
//   Hessians, no definiteness projection); solve (M / h^2 - K) dx = f by conjugate gradients
//   with the diagonal preconditioner (Eigen::ConjugateGradient: relative tolerance 1e-5,
//   300 iterations); x = y + dx; v = (x - x0) / h.
//
// Layout: the global matrix is block-sparse with 3x3 blocks (BSR) over the vertex adjacency of
// all stencils; one thread per element computes the element's gradient and Hessian blocks by
// forward-mode differentiation over vertex pairs (6 seeded coordinates) and adds them with
// atomics. Vectors are FP32, inner products FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "api_internal.h"
#include "devbuf.h"
#include "device_common.cuh"
#include "layout.h"
#include "state.h"

namespace spgx {

struct ImplicitTables {
    const int4 *idx;    // per element: internal vertex ids (-1 padded)
    const int4 *info;   // per element: {type, param offset, stencil size, 0}
    const float *prm;   // parameters in the spgx.h layouts
    const int *eblk;    // per element: S x S block positions in the BSR values (row-major)
    const int *row_ptr;  // BSR rows (internal vertices)
    const int *col;      // BSR block columns
    float *val;          // BSR values, 9 per block (row-major)
    const int *diag;     // per vertex: position of its diagonal block
};

__device__ __forceinline__ void atomic_block(float *val, int blk, const float H[9])
{
    float *b = val + size_t(blk) * 9;
#pragma unroll
    for (int k = 0; k < 9; ++k) atomicAdd(b + k, H[k]);
}

__device__ __forceinline__ void atomic_force(float4 *f, int v, float gx, float gy, float gz)
{
    atomicAdd(&f[v].x, -gx);
    atomicAdd(&f[v].y, -gy);
    atomicAdd(&f[v].z, -gz);
}

// Gradient and Hessian blocks of one element at the current positions, added to the forces
// (f -= grad) and to the matrix (val += hess).
template <int S>
__device__ void assemble_element(const ImplicitTables &T, const float4 *__restrict__ pos, float4 *force, int e,
                                 int4 ix, int4 info)
{
    const int iv[4] = {ix.x, ix.y, ix.z, ix.w};
    const float *prm = T.prm + info.y;
    const int type = info.x;
    const int *eb = T.eblk + size_t(e) * 16;
    const float4 b0 = pos[2 * iv[0]], d0 = pos[2 * iv[0] + 1];
    Vec3<float> p[S];
#pragma unroll
    for (int j = 0; j < S; ++j) {
        const float4 b = pos[2 * iv[j]], d = pos[2 * iv[j] + 1];
        p[j] = mk((b.x - b0.x) + (d.x - d0.x), (b.y - b0.y) + (d.y - d0.y), (b.z - b0.z) + (d.z - d0.z));
    }
    if (type == SPGX_ENERGY_QUADRATIC_BENDING) {
        // C = sum_s c_s x_s (linear): grad_a = k c_a C, hess_ab = k c_a c_b I.
        Vec3<float> C = mk(0.f, 0.f, 0.f);
#pragma unroll
        for (int s = 0; s < S; ++s) C = C + prm[s] * p[s];
        const float k = prm[4];
#pragma unroll
        for (int a = 0; a < S; ++a) {
            atomic_force(force, iv[a], k * prm[a] * C.x, k * prm[a] * C.y, k * prm[a] * C.z);
#pragma unroll
            for (int b = 0; b < S; ++b) {
                const float s = k * prm[a] * prm[b];
                const float H[9] = {s, 0.f, 0.f, 0.f, s, 0.f, 0.f, 0.f, s};
                atomic_block(T.val, eb[a * S + b], H);
            }
        }
        return;
    }
    // Vertex pairs (a, b), a < b: 6 seeded coordinates give blocks (a,a), (a,b), (b,b). The
    // diagonal block and gradient of a vertex are taken from one pair only: (a, a+1), and for
    // the last vertex (S-2, S-1).
#pragma unroll
    for (int a = 0; a < S; ++a)
#pragma unroll
        for (int b = a + 1; b < S; ++b) {
            V3A<float, 6> q[S];
            seed_positions<float, S, 6>(p, a, q, b);
            const VAD<float, 6> E = energy_ad(type, q, prm);
            float Hab[9], Hba[9];
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    Hab[3 * r + c] = E.h[hidx<6>(r, 3 + c)];
                    Hba[3 * c + r] = Hab[3 * r + c];
                }
            atomic_block(T.val, eb[a * S + b], Hab);
            atomic_block(T.val, eb[b * S + a], Hba);
            const bool diag_a = b == a + 1;
            const bool diag_b = a == S - 2 && b == S - 1;
            if (diag_a) {
                float H[9];
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c) H[3 * r + c] = E.h[r <= c ? hidx<6>(r, c) : hidx<6>(c, r)];
                atomic_block(T.val, eb[a * S + a], H);
                atomic_force(force, iv[a], E.g[0], E.g[1], E.g[2]);
            }
            if (diag_b) {
                float H[9];
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        H[3 * r + c] = E.h[r <= c ? hidx<6>(3 + r, 3 + c) : hidx<6>(3 + c, 3 + r)];
                atomic_block(T.val, eb[b * S + b], H);
                atomic_force(force, iv[b], E.g[3], E.g[4], E.g[5]);
            }
        }
}

__global__ void __launch_bounds__(128) implicit_assemble_kernel(ImplicitTables T, const float4 *__restrict__ pos,
                                                                float4 *force, int n_elem)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_elem) return;
    const int4 ix = __ldg(T.idx + e);
    const int4 info = __ldg(T.info + e);
    const float *prm = T.prm + info.y;
    switch (info.z) {
    case 1: {
        const int v = ix.x;
        if (info.x == SPGX_ENERGY_STATIC_LOAD) {  // E = -k d . x: force k d, no Hessian
            atomic_force(force, v, -prm[0] * prm[1], -prm[0] * prm[2], -prm[0] * prm[3]);
            return;
        }
        // Anchor: 1/2 k |x - a|^2 on the anchor-relative position.
        const float4 b = pos[2 * v], d = pos[2 * v + 1];
        const float xa[3] = {(b.x - prm[0]) + d.x, (b.y - prm[1]) + d.y, (b.z - prm[2]) + d.z};
        const float k = prm[3];
        atomic_force(force, v, k * xa[0], k * xa[1], k * xa[2]);
        const float H[9] = {k, 0.f, 0.f, 0.f, k, 0.f, 0.f, 0.f, k};
        atomic_block(T.val, T.eblk[size_t(e) * 16], H);
        return;
    }
    case 2: assemble_element<2>(T, pos, force, e, ix, info); break;
    case 3: assemble_element<3>(T, pos, force, e, ix, info); break;
    default: assemble_element<4>(T, pos, force, e, ix, info); break;
    }
}

// x0 = x (rebased: base = fl(x), dold = the exact remainder), y = x + h v as the delta, and the
// forces initialised to M g.
__global__ void implicit_predict_kernel(float4 *pos, float4 *dold, const float4 *vel, const float *mass, float4 *force,
                                       int nv, float h, float gx, float gy, float gz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float4 b = pos[2 * i], d = pos[2 * i + 1];
    const float4 v = vel[i];
    float s[3], r[3];
    const float bb[3] = {b.x, b.y, b.z}, dd[3] = {d.x, d.y, d.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        s[k] = bb[k] + dd[k];
        const float t = s[k] - bb[k];
        r[k] = (bb[k] - (s[k] - t)) + (dd[k] - t);
    }
    pos[2 * i] = make_float4(s[0], s[1], s[2], b.w);
    pos[2 * i + 1] = make_float4(r[0] + h * v.x, r[1] + h * v.y, r[2] + h * v.z, 0.f);
    dold[i] = make_float4(r[0], r[1], r[2], 0.f);
    const float m = mass[i];
    force[i] = make_float4(m * gx, m * gy, m * gz, 0.f);
}

// The mass term M / h^2 on the diagonal blocks and the diagonal preconditioner 1 / A_ii.
__global__ void implicit_mass_kernel(ImplicitTables T, const float *mass, int nv, float invh2, float4 *dinv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    float *b = T.val + size_t(T.diag[i]) * 9;
    const float m = mass[i] * invh2;
    b[0] += m;
    b[4] += m;
    b[8] += m;
    // Eigen's DiagonalPreconditioner: 1 / A_ii, or 1 where A_ii is 0.
    dinv[i] = make_float4(b[0] != 0.f ? 1.f / b[0] : 1.f, b[4] != 0.f ? 1.f / b[4] : 1.f,
                          b[8] != 0.f ? 1.f / b[8] : 1.f, 0.f);
}

__device__ __forceinline__ void block_reduce_add(double v, double *out)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __shared__ double part[32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) part[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < (blockDim.x + 31) / 32; ++k) s += part[k];
        atomicAdd(out, s);
    }
}

// Ap = A p (one thread per block row) and dots[0] += p . Ap.
__global__ void implicit_spmv_kernel(ImplicitTables T, const float4 *__restrict__ p, float4 *Ap, int nv, double *dots)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double pap = 0.0;
    if (i < nv) {
        float y0 = 0.f, y1 = 0.f, y2 = 0.f;
        for (int k = __ldg(T.row_ptr + i); k < __ldg(T.row_ptr + i + 1); ++k) {
            const float *b = T.val + size_t(k) * 9;
            const float4 x = p[__ldg(T.col + k)];
            y0 += b[0] * x.x + b[1] * x.y + b[2] * x.z;
            y1 += b[3] * x.x + b[4] * x.y + b[5] * x.z;
            y2 += b[6] * x.x + b[7] * x.y + b[8] * x.z;
        }
        Ap[i] = make_float4(y0, y1, y2, 0.f);
        const float4 pi = p[i];
        pap = double(pi.x) * y0 + double(pi.y) * y1 + double(pi.z) * y2;
    }
    block_reduce_add(pap, dots);
}

// CG start with x = 0: r = b, z = D^-1 r, p = z; dots[1] += r.r, dots[2] += r.z.
__global__ void implicit_cg_init_kernel(const float4 *b, const float4 *dinv, float4 *x, float4 *r, float4 *z,
                                       float4 *p, int nv, double *dots)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0, rz = 0.0;
    if (i < nv) {
        const float4 ri = b[i], di = dinv[i];
        const float4 zi = make_float4(ri.x * di.x, ri.y * di.y, ri.z * di.z, 0.f);
        x[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        r[i] = make_float4(ri.x, ri.y, ri.z, 0.f);
        z[i] = zi;
        p[i] = zi;
        rr = double(ri.x) * ri.x + double(ri.y) * ri.y + double(ri.z) * ri.z;
        rz = double(ri.x) * zi.x + double(ri.y) * zi.y + double(ri.z) * zi.z;
    }
    block_reduce_add(rr, dots + 1);
    block_reduce_add(rz, dots + 2);
}

// x += alpha p; r -= alpha Ap; z = D^-1 r; dots[1] += r.r, dots[2] += r.z (alpha = rz / pAp).
__global__ void implicit_cg_update_kernel(float4 *x, float4 *r, float4 *z, const float4 *p, const float4 *Ap,
                                         const float4 *dinv, int nv, const double *prev, double *dots)
{
    const float alpha = static_cast<float>(prev[2] / prev[0]);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0, rz = 0.0;
    if (i < nv) {
        const float4 pi = p[i], api = Ap[i], di = dinv[i];
        float4 xi = x[i], ri = r[i];
        xi.x += alpha * pi.x;
        xi.y += alpha * pi.y;
        xi.z += alpha * pi.z;
        ri.x -= alpha * api.x;
        ri.y -= alpha * api.y;
        ri.z -= alpha * api.z;
        x[i] = xi;
        r[i] = ri;
        const float4 zi = make_float4(ri.x * di.x, ri.y * di.y, ri.z * di.z, 0.f);
        z[i] = zi;
        rr = double(ri.x) * ri.x + double(ri.y) * ri.y + double(ri.z) * ri.z;
        rz = double(ri.x) * zi.x + double(ri.y) * zi.y + double(ri.z) * zi.z;
    }
    block_reduce_add(rr, dots + 1);
    block_reduce_add(rz, dots + 2);
}

// p = z + beta p, beta = rz_new / rz_old.
__global__ void implicit_cg_direction_kernel(float4 *p, const float4 *z, int nv, const double *prev, const double *cur)
{
    const float beta = static_cast<float>(cur[2] / prev[2]);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float4 zi = z[i], pi = p[i];
    p[i] = make_float4(zi.x + beta * pi.x, zi.y + beta * pi.y, zi.z + beta * pi.z, 0.f);
}

// x = y + dx (the delta holds y).
__global__ void implicit_apply_kernel(float4 *pos, const float4 *dx, int nv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    float4 d = pos[2 * i + 1];
    const float4 a = dx[i];
    d.x += a.x;
    d.y += a.y;
    d.z += a.z;
    pos[2 * i + 1] = d;
}

static int grid_of(int n, int t = 256) { return (n + t - 1) / t; }

struct ImplicitSolver {
    SceneLayout L;
    spgx_implicit_params P{};
    int device{0};
    cudaStream_t stream{nullptr};
    cudaEvent_t ev0{nullptr}, ev1{nullptr};
    ParticleState X;
    DevBuf d_idx, d_info, d_prm, d_eblk, d_row, d_col, d_val, d_diag, d_mass;
    DevBuf d_force, d_dinv, d_x, d_r, d_z, d_p, d_Ap, d_dots;
    HostBuf h_dots;
    ImplicitTables T{};
    int n_elem{0}, nnzb{0};

    ~ImplicitSolver()
    {
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
    }

    static spgx_status check_params(const spgx_implicit_params *p)
    {
        if (!p || !(p->dt > 0) || p->substeps < 1 || !(p->cg_threshold >= 0) || p->cg_max_iterations < 0) {
            set_error("invalid implicit Euler parameters");
            return SPGX_ERR_INVALID_ARG;
        }
        return SPGX_OK;
    }

    spgx_status init(const spgx_scene_desc *scene, const spgx_implicit_params *params)
    {
        std::string err;
        SPGX_TRY_STATUS(check_params(params));
        const spgx_status st = build_scene_layout(scene, false, L, err);
        if (st != SPGX_OK) {
            set_error(err);
            return st;
        }
        P = *params;
        SPGX_TRY_STATUS(select_device(P.device));
        device = P.device;
        SPGX_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        SPGX_CUDA(cudaEventCreate(&ev0));
        SPGX_CUDA(cudaEventCreate(&ev1));
        SPGX_TRY_STATUS(X.init(L));
        // Element list over every energy (internal vertex ids) and the block pattern.
        const int nv = L.nv;
        std::vector<I4> idx, info;
        std::vector<float> prm;
        std::vector<std::vector<int32_t>> nb(nv);
        for (int v = 0; v < nv; ++v) nb[v].push_back(v);
        for (int o = 0; o < scene->n_objects; ++o) {
            const auto &ob = scene->objects[o];
            const int vb = L.objects[o].vertex_base;
            for (int e = 0; e < ob.n_energies; ++e) {
                const auto &E = ob.energies[e];
                const int S = stencil_size(E.type), Pc = param_count(E.type);
                for (int s = 0; s < E.n_stencils; ++s) {
                    int iv[4] = {-1, -1, -1, -1};
                    for (int k = 0; k < S; ++k) iv[k] = L.ext2int[vb + E.stencils[int64_t(s) * S + k]];
                    idx.push_back({iv[0], iv[1], iv[2], iv[3]});
                    info.push_back({E.type, static_cast<int32_t>(prm.size()), S, 0});
                    for (int k = 0; k < Pc; ++k) prm.push_back(static_cast<float>(E.params[int64_t(s) * Pc + k]));
                    for (int a = 0; a < S; ++a)
                        for (int b = 0; b < S; ++b)
                            if (a != b) nb[iv[a]].push_back(iv[b]);
                }
            }
        }
        n_elem = static_cast<int>(idx.size());
        std::vector<int32_t> row(nv + 1, 0), col, diag(nv);
        for (int v = 0; v < nv; ++v) {
            auto &r = nb[v];
            std::sort(r.begin(), r.end());
            r.erase(std::unique(r.begin(), r.end()), r.end());
            for (int c : r) {
                if (c == v) diag[v] = static_cast<int32_t>(col.size());
                col.push_back(c);
            }
            row[v + 1] = static_cast<int32_t>(col.size());
        }
        nnzb = static_cast<int>(col.size());
        std::vector<int32_t> eblk(size_t(std::max(1, n_elem)) * 16, 0);
        for (int e = 0; e < n_elem; ++e) {
            const int iv[4] = {idx[e].x, idx[e].y, idx[e].z, idx[e].w};
            const int S = info[e].z;
            for (int a = 0; a < S; ++a)
                for (int b = 0; b < S; ++b) {
                    const auto first = col.begin() + row[iv[a]], last = col.begin() + row[iv[a] + 1];
                    eblk[size_t(e) * 16 + a * S + b] = static_cast<int32_t>(std::lower_bound(first, last, iv[b]) - col.begin());
                }
        }
        if (idx.empty()) {
            idx.push_back({0, -1, -1, -1});
            info.push_back({0, 0, 0, 0});
        }
        if (prm.empty()) prm.push_back(0.f);
        if (col.empty()) col.push_back(0);
        SPGX_TRY_STATUS(d_idx.upload(idx));
        SPGX_TRY_STATUS(d_info.upload(info));
        SPGX_TRY_STATUS(d_prm.upload(prm));
        SPGX_TRY_STATUS(d_eblk.upload(eblk));
        SPGX_TRY_STATUS(d_row.upload(row));
        SPGX_TRY_STATUS(d_col.upload(col));
        SPGX_TRY_STATUS(d_diag.upload(diag.empty() ? std::vector<int32_t>{0} : diag));
        SPGX_TRY_STATUS(d_mass.upload(L.mass.empty() ? std::vector<float>{0.f} : L.mass));
        SPGX_TRY_STATUS(d_val.alloc(size_t(std::max(1, nnzb)) * 9 * sizeof(float)));
        const size_t vec = size_t(std::max(1, nv)) * sizeof(float4);
        for (DevBuf *b : {&d_force, &d_dinv, &d_x, &d_r, &d_z, &d_p, &d_Ap}) SPGX_TRY_STATUS(b->alloc(vec));
        SPGX_TRY_STATUS(d_dots.alloc(size_t(2) * 3 * sizeof(double)));
        SPGX_TRY_STATUS(h_dots.alloc(size_t(2) * 3 * sizeof(double)));
        T = ImplicitTables{d_idx.as<int4>(), d_info.as<int4>(), d_prm.as<float>(), d_eblk.as<int>(), d_row.as<int>(),
                           d_col.as<int>(), d_val.as<float>(), d_diag.as<int>()};
        return SPGX_OK;
    }

    // One CG solve of A dx = f (ImplicitEulerBase::solveLinearSystem, implicitEulerBase.cpp:227-239)
    // with Eigen::ConjugateGradient's stopping rule |r|^2 < tol^2 |b|^2.
    spgx_status cg(int &iterations, double &rel_residual)
    {
        const int nv = L.nv;
        double *dots = d_dots.as<double>();  // two sets of {pAp, rr, rz}: [0..2] previous, [3..5] current
        double *hd = h_dots.as<double>();
        SPGX_CUDA(cudaMemsetAsync(dots, 0, 6 * sizeof(double), stream));
        implicit_cg_init_kernel<<<grid_of(nv), 256, 0, stream>>>(d_force.as<float4>(), d_dinv.as<float4>(),
                                                                 d_x.as<float4>(), d_r.as<float4>(), d_z.as<float4>(),
                                                                 d_p.as<float4>(), nv, dots);
        SPGX_CUDA(cudaMemcpyAsync(hd, dots, 3 * sizeof(double), cudaMemcpyDeviceToHost, stream));
        SPGX_CUDA(cudaStreamSynchronize(stream));
        const double rhs2 = hd[1];
        iterations = 0;
        rel_residual = 0.0;
        if (rhs2 == 0.0) return SPGX_OK;  // x = 0
        const double thr2 = std::max(P.cg_threshold * P.cg_threshold * rhs2, 1e-300);
        double rr = rhs2;
        double *prev = dots, *cur = dots + 3;
        while (rr >= thr2 && iterations < P.cg_max_iterations) {
            // prev = {pAp, rr, rz} of this iteration's start
            SPGX_CUDA(cudaMemsetAsync(prev, 0, sizeof(double), stream));
            implicit_spmv_kernel<<<grid_of(nv), 256, 0, stream>>>(T, d_p.as<float4>(), d_Ap.as<float4>(), nv, prev);
            SPGX_CUDA(cudaMemsetAsync(cur, 0, 3 * sizeof(double), stream));
            implicit_cg_update_kernel<<<grid_of(nv), 256, 0, stream>>>(d_x.as<float4>(), d_r.as<float4>(),
                                                                      d_z.as<float4>(), d_p.as<float4>(),
                                                                      d_Ap.as<float4>(), d_dinv.as<float4>(), nv,
                                                                      prev, cur);
            implicit_cg_direction_kernel<<<grid_of(nv), 256, 0, stream>>>(d_p.as<float4>(), d_z.as<float4>(), nv,
                                                                          prev, cur);
            SPGX_CUDA(cudaMemcpyAsync(hd, cur, 3 * sizeof(double), cudaMemcpyDeviceToHost, stream));
            SPGX_CUDA(cudaStreamSynchronize(stream));
            rr = hd[1];
            ++iterations;
            std::swap(prev, cur);
        }
        rel_residual = std::sqrt(rr / rhs2);
        return SPGX_OK;
    }

    spgx_status step(spgx_step_stats *stats)
    {
        SPGX_TRY_STATUS(X.upload_if_dirty(stream));
        X.mark_device_advanced();
        spgx_step_stats st{};
        st.converged = 1;
        const int nv = L.nv;
        const double h = P.dt / P.substeps;
        SPGX_CUDA(cudaEventRecord(ev0, stream));
        for (int s = 0; s < P.substeps && nv > 0; ++s) {
            implicit_predict_kernel<<<grid_of(nv), 256, 0, stream>>>(X.pos(), X.dold(), X.vel(), d_mass.as<float>(),
                                                                     d_force.as<float4>(), nv, float(h),
                                                                     float(P.gravity[0]), float(P.gravity[1]),
                                                                     float(P.gravity[2]));
            SPGX_CUDA(cudaMemsetAsync(d_val.as<float>(), 0, size_t(std::max(1, nnzb)) * 9 * sizeof(float), stream));
            if (n_elem > 0)
                implicit_assemble_kernel<<<grid_of(n_elem, 128), 128, 0, stream>>>(T, X.pos(), d_force.as<float4>(),
                                                                                  n_elem);
            implicit_mass_kernel<<<grid_of(nv), 256, 0, stream>>>(T, d_mass.as<float>(), nv, float(1.0 / (h * h)),
                                                                  d_dinv.as<float4>());
            SPGX_CUDA(cudaGetLastError());
            int its = 0;
            double rel = 0.0;
            SPGX_TRY_STATUS(cg(its, rel));
            st.iterations += its;
            st.residual_final = rel;
            if (rel > P.cg_threshold) st.converged = 0;
            implicit_apply_kernel<<<grid_of(nv), 256, 0, stream>>>(X.pos(), d_x.as<float4>(), nv);
            launch_end_substep(X, h, stream);
        }
        SPGX_CUDA(cudaEventRecord(ev1, stream));
        SPGX_CUDA(cudaGetLastError());
        SPGX_CUDA(cudaStreamSynchronize(stream));
        float ms = 0.f;
        SPGX_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        st.device_ms = ms;
        if (stats) *stats = st;
        return SPGX_OK;
    }
};

}  // namespace spgx

// =======================================================================================
// C ABI

struct spgx_implicit {
    std::unique_ptr<spgx::ImplicitSolver> s;
};

extern "C" {

void spgx_implicit_params_default(spgx_implicit_params *p)
{
    if (!p) return;
    *p = spgx_implicit_params{};
    p->dt = 0.01;
    p->substeps = 1;
    p->gravity[0] = 0.0;
    p->gravity[1] = -9.8;
    p->gravity[2] = 0.0;
    p->cg_threshold = 1e-5;
    p->cg_max_iterations = 300;
    p->device = 0;
}

spgx_status spgx_implicit_create(const spgx_scene_desc *scene, const spgx_implicit_params *params, spgx_implicit **out)
{
    SPGX_GUARD_BEGIN
    if (!out) {
        spgx::set_error("out is NULL");
        return SPGX_ERR_INVALID_ARG;
    }
    *out = nullptr;
    auto h = std::make_unique<spgx_implicit>();
    h->s = std::make_unique<spgx::ImplicitSolver>();
    SPGX_TRY_STATUS(h->s->init(scene, params));
    *out = h.release();
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_implicit_destroy(spgx_implicit *h)
{
    SPGX_GUARD_BEGIN
    if (h) {
        cudaSetDevice(h->s->device);
        delete h;
    }
    return SPGX_OK;
    SPGX_GUARD_END
}

#define SPGX_IHANDLE(h)                                \
    if (!(h)) {                                        \
        spgx::set_error("NULL implicit solver handle"); \
        return SPGX_ERR_INVALID_ARG;                   \
    }                                                  \
    SPGX_CUDA(cudaSetDevice((h)->s->device))

spgx_status spgx_implicit_step(spgx_implicit *h, spgx_step_stats *stats)
{
    SPGX_GUARD_BEGIN
    SPGX_IHANDLE(h);
    return h->s->step(stats);
    SPGX_GUARD_END
}

spgx_status spgx_implicit_get_state(spgx_implicit *h, int32_t object, double *x, double *v)
{
    SPGX_GUARD_BEGIN
    SPGX_IHANDLE(h);
    return h->s->X.get(h->s->L, object, x, v, h->s->stream);
    SPGX_GUARD_END
}

spgx_status spgx_implicit_set_state(spgx_implicit *h, int32_t object, const double *x, const double *v)
{
    SPGX_GUARD_BEGIN
    SPGX_IHANDLE(h);
    return h->s->X.set(h->s->L, object, x, v, h->s->stream);
    SPGX_GUARD_END
}

spgx_status spgx_implicit_reset(spgx_implicit *h)
{
    SPGX_GUARD_BEGIN
    SPGX_IHANDLE(h);
    return h->s->X.reset(h->s->L, h->s->stream);
    SPGX_GUARD_END
}

}  // extern "C"
