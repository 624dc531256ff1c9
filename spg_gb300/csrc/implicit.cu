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
// atomics. Assembly, parameters and the CG run in FP64 (the positions stay FP32 base + delta):
// a flat cloth at rest has no transverse stiffness, and FP32 rounding of 1 - L0 / |x1 - x0|
// would add some of the order of the M / h^2 term and change the solution. This solver is off
// the VBD hot path, so FP64's lower rate is acceptable here.
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
    const int4 *idx;     // per element: internal vertex ids (-1 padded)
    const int4 *info;    // per element: {type, param offset, stencil size, 0}
    const double *prm;   // parameters in the spgx.h layouts
    const int *eblk;     // per element: S x S block positions in the BSR values (row-major)
    const int *row_ptr;  // BSR rows (internal vertices)
    const int *col;      // BSR block columns
    double *val;         // BSR values, 9 per block (row-major)
    const int *diag;     // per vertex: position of its diagonal block
};

// Vectors over the vertices: 3 doubles per vertex.
__device__ __forceinline__ void atomic_block(double *val, int blk, const double H[9])
{
    double *b = val + size_t(blk) * 9;
#pragma unroll
    for (int k = 0; k < 9; ++k) atomicAdd(b + k, H[k]);
}

__device__ __forceinline__ void atomic_force(double *f, int v, double gx, double gy, double gz)
{
    atomicAdd(f + 3 * v, -gx);
    atomicAdd(f + 3 * v + 1, -gy);
    atomicAdd(f + 3 * v + 2, -gz);
}

// Position of vertex j relative to (b0, d0), in FP64 from the FP32 base/delta pairs.
__device__ __forceinline__ Vec3<double> rel64(const float4 *pos, int j, float4 b0, float4 d0)
{
    const float4 b = pos[2 * j], d = pos[2 * j + 1];
    return mk((double(b.x) - b0.x) + (double(d.x) - d0.x), (double(b.y) - b0.y) + (double(d.y) - d0.y),
              (double(b.z) - b0.z) + (double(d.z) - d0.z));
}

// Gradient and Hessian blocks of one element at the current positions, added to the forces
// (f -= grad) and to the matrix (val += hess).
template <int S>
__device__ void assemble_element(const ImplicitTables &T, const float4 *__restrict__ pos, double *force, int e,
                                 int4 ix, int4 info)
{
    const int iv[4] = {ix.x, ix.y, ix.z, ix.w};
    const double *prm = T.prm + info.y;
    const int type = info.x;
    const int *eb = T.eblk + size_t(e) * 16;
    const float4 b0 = pos[2 * iv[0]], d0 = pos[2 * iv[0] + 1];
    Vec3<double> p[S];
#pragma unroll
    for (int j = 0; j < S; ++j) p[j] = rel64(pos, iv[j], b0, d0);
    if (type == SPGX_ENERGY_QUADRATIC_BENDING) {
        // C = sum_s c_s x_s (linear): grad_a = k c_a C, hess_ab = k c_a c_b I.
        Vec3<double> C = mk(0.0, 0.0, 0.0);
#pragma unroll
        for (int s = 0; s < S; ++s) C = C + prm[s] * p[s];
        const double k = prm[4];
#pragma unroll
        for (int a = 0; a < S; ++a) {
            atomic_force(force, iv[a], k * prm[a] * C.x, k * prm[a] * C.y, k * prm[a] * C.z);
#pragma unroll
            for (int b = 0; b < S; ++b) {
                const double s = k * prm[a] * prm[b];
                const double H[9] = {s, 0.0, 0.0, 0.0, s, 0.0, 0.0, 0.0, s};
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
            V3A<double, 6> q[S];
            seed_positions<double, S, 6>(p, a, q, b);
            const VAD<double, 6> E = energy_ad(type, q, prm);
            double Hab[9], Hba[9];
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
                double H[9];
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c) H[3 * r + c] = E.h[r <= c ? hidx<6>(r, c) : hidx<6>(c, r)];
                atomic_block(T.val, eb[a * S + a], H);
                atomic_force(force, iv[a], E.g[0], E.g[1], E.g[2]);
            }
            if (diag_b) {
                double H[9];
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
                                                                double *force, int n_elem)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_elem) return;
    const int4 ix = __ldg(T.idx + e);
    const int4 info = __ldg(T.info + e);
    const double *prm = T.prm + info.y;
    switch (info.z) {
    case 1: {
        const int v = ix.x;
        if (info.x == SPGX_ENERGY_STATIC_LOAD) {  // E = -k d . x: force k d, no Hessian
            atomic_force(force, v, -prm[0] * prm[1], -prm[0] * prm[2], -prm[0] * prm[3]);
            return;
        }
        // Anchor: 1/2 k |x - a|^2 on the anchor-relative position.
        const float4 b = pos[2 * v], d = pos[2 * v + 1];
        const double xa[3] = {(double(b.x) - prm[0]) + d.x, (double(b.y) - prm[1]) + d.y, (double(b.z) - prm[2]) + d.z};
        const double k = prm[3];
        atomic_force(force, v, k * xa[0], k * xa[1], k * xa[2]);
        const double H[9] = {k, 0.0, 0.0, 0.0, k, 0.0, 0.0, 0.0, k};
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
__global__ void implicit_predict_kernel(float4 *pos, float4 *dold, const float4 *vel, const float *mass, double *force,
                                       int nv, float h, double gx, double gy, double gz)
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
    const double m = mass[i];
    force[3 * i] = m * gx;
    force[3 * i + 1] = m * gy;
    force[3 * i + 2] = m * gz;
}

// The mass term M / h^2 on the diagonal blocks and the diagonal preconditioner 1 / A_ii.
__global__ void implicit_mass_kernel(ImplicitTables T, const float *mass, int nv, double invh2, double *dinv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    double *b = T.val + size_t(T.diag[i]) * 9;
    const double m = double(mass[i]) * invh2;
    b[0] += m;
    b[4] += m;
    b[8] += m;
    // Eigen's DiagonalPreconditioner: 1 / A_ii, or 1 where A_ii is 0.
    dinv[3 * i] = b[0] != 0.0 ? 1.0 / b[0] : 1.0;
    dinv[3 * i + 1] = b[4] != 0.0 ? 1.0 / b[4] : 1.0;
    dinv[3 * i + 2] = b[8] != 0.0 ? 1.0 / b[8] : 1.0;
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
__global__ void implicit_spmv_kernel(ImplicitTables T, const double *__restrict__ p, double *Ap, int nv, double *dots)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double pap = 0.0;
    if (i < nv) {
        double y0 = 0.0, y1 = 0.0, y2 = 0.0;
        for (int k = __ldg(T.row_ptr + i); k < __ldg(T.row_ptr + i + 1); ++k) {
            const double *bl = T.val + size_t(k) * 9;
            const double *x = p + 3 * size_t(__ldg(T.col + k));
            y0 += bl[0] * x[0] + bl[1] * x[1] + bl[2] * x[2];
            y1 += bl[3] * x[0] + bl[4] * x[1] + bl[5] * x[2];
            y2 += bl[6] * x[0] + bl[7] * x[1] + bl[8] * x[2];
        }
        Ap[3 * i] = y0;
        Ap[3 * i + 1] = y1;
        Ap[3 * i + 2] = y2;
        pap = p[3 * i] * y0 + p[3 * i + 1] * y1 + p[3 * i + 2] * y2;
    }
    block_reduce_add(pap, dots);
}

// CG start with x = 0: r = b, z = D^-1 r, p = z; dots[1] += r.r, dots[2] += r.z (per component).
__global__ void implicit_cg_init_kernel(const double *b, const double *dinv, double *x, double *r, double *z,
                                       double *p, int n, double *dots)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0, rz = 0.0;
    if (i < n) {
        const double ri = b[i], zi = ri * dinv[i];
        x[i] = 0.0;
        r[i] = ri;
        z[i] = zi;
        p[i] = zi;
        rr = ri * ri;
        rz = ri * zi;
    }
    block_reduce_add(rr, dots + 1);
    block_reduce_add(rz, dots + 2);
}

// x += alpha p; r -= alpha Ap; z = D^-1 r; dots[1] += r.r, dots[2] += r.z (alpha = rz / pAp).
__global__ void implicit_cg_update_kernel(double *x, double *r, double *z, const double *p, const double *Ap,
                                         const double *dinv, int n, const double *prev, double *dots)
{
    const double alpha = prev[2] / prev[0];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0, rz = 0.0;
    if (i < n) {
        x[i] += alpha * p[i];
        const double ri = r[i] - alpha * Ap[i];
        r[i] = ri;
        const double zi = ri * dinv[i];
        z[i] = zi;
        rr = ri * ri;
        rz = ri * zi;
    }
    block_reduce_add(rr, dots + 1);
    block_reduce_add(rz, dots + 2);
}

// p = z + beta p, beta = rz_new / rz_old.
__global__ void implicit_cg_direction_kernel(double *p, const double *z, int n, const double *prev, const double *cur)
{
    const double beta = cur[2] / prev[2];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    p[i] = z[i] + beta * p[i];
}

// x = y + dx (the delta holds y).
__global__ void implicit_apply_kernel(float4 *pos, const double *dx, int nv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    float4 d = pos[2 * i + 1];
    d.x = static_cast<float>(d.x + dx[3 * i]);
    d.y = static_cast<float>(d.y + dx[3 * i + 1]);
    d.z = static_cast<float>(d.z + dx[3 * i + 2]);
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
        std::vector<double> prm;
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
                    for (int k = 0; k < Pc; ++k) prm.push_back(E.params[int64_t(s) * Pc + k]);
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
        if (prm.empty()) prm.push_back(0.0);
        if (col.empty()) col.push_back(0);
        SPGX_TRY_STATUS(d_idx.upload(idx));
        SPGX_TRY_STATUS(d_info.upload(info));
        SPGX_TRY_STATUS(d_prm.upload(prm));
        SPGX_TRY_STATUS(d_eblk.upload(eblk));
        SPGX_TRY_STATUS(d_row.upload(row));
        SPGX_TRY_STATUS(d_col.upload(col));
        SPGX_TRY_STATUS(d_diag.upload(diag.empty() ? std::vector<int32_t>{0} : diag));
        SPGX_TRY_STATUS(d_mass.upload(L.mass.empty() ? std::vector<float>{0.f} : L.mass));
        SPGX_TRY_STATUS(d_val.alloc(size_t(std::max(1, nnzb)) * 9 * sizeof(double)));
        const size_t vec = size_t(std::max(1, nv)) * 3 * sizeof(double);
        for (DevBuf *b : {&d_force, &d_dinv, &d_x, &d_r, &d_z, &d_p, &d_Ap}) SPGX_TRY_STATUS(b->alloc(vec));
        SPGX_TRY_STATUS(d_dots.alloc(size_t(2) * 3 * sizeof(double)));
        SPGX_TRY_STATUS(h_dots.alloc(size_t(2) * 3 * sizeof(double)));
        T = ImplicitTables{d_idx.as<int4>(), d_info.as<int4>(), d_prm.as<double>(), d_eblk.as<int>(), d_row.as<int>(),
                           d_col.as<int>(), d_val.as<double>(), d_diag.as<int>()};
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
        const int n = 3 * nv;
        implicit_cg_init_kernel<<<grid_of(n), 256, 0, stream>>>(d_force.as<double>(), d_dinv.as<double>(),
                                                                d_x.as<double>(), d_r.as<double>(), d_z.as<double>(),
                                                                d_p.as<double>(), n, dots);
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
            implicit_spmv_kernel<<<grid_of(nv), 256, 0, stream>>>(T, d_p.as<double>(), d_Ap.as<double>(), nv, prev);
            SPGX_CUDA(cudaMemsetAsync(cur, 0, 3 * sizeof(double), stream));
            implicit_cg_update_kernel<<<grid_of(n), 256, 0, stream>>>(d_x.as<double>(), d_r.as<double>(),
                                                                     d_z.as<double>(), d_p.as<double>(),
                                                                     d_Ap.as<double>(), d_dinv.as<double>(), n, prev,
                                                                     cur);
            implicit_cg_direction_kernel<<<grid_of(n), 256, 0, stream>>>(d_p.as<double>(), d_z.as<double>(), n, prev,
                                                                         cur);
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
                                                                     d_force.as<double>(), nv, float(h), P.gravity[0],
                                                                     P.gravity[1], P.gravity[2]);
            SPGX_CUDA(cudaMemsetAsync(d_val.as<double>(), 0, size_t(std::max(1, nnzb)) * 9 * sizeof(double), stream));
            if (n_elem > 0)
                implicit_assemble_kernel<<<grid_of(n_elem, 128), 128, 0, stream>>>(T, X.pos(), d_force.as<double>(),
                                                                                  n_elem);
            implicit_mass_kernel<<<grid_of(nv), 256, 0, stream>>>(T, d_mass.as<float>(), nv, 1.0 / (h * h),
                                                                  d_dinv.as<double>());
            SPGX_CUDA(cudaGetLastError());
            int its = 0;
            double rel = 0.0;
            SPGX_TRY_STATUS(cg(its, rel));
            st.iterations += its;
            st.residual_final = rel;
            if (rel > P.cg_threshold) st.converged = 0;
            implicit_apply_kernel<<<grid_of(nv), 256, 0, stream>>>(X.pos(), d_x.as<double>(), nv);
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
