// adjoint.cu -- variable-rate ADI (a rate D per cell) and the gradient of a
// field loss by reverse-mode differentiation, with checkpoints.
//
// The reference has no variable-rate ADI and no gradient code.  The step is
// defined from HAL's variable-rate explicit stencil Internal::Diffusion2(...,
// pDiffRatesX, pDiffRatesY, ...) (src/Pde/PDEequations.cpp:199-230): the
// face between cells j and j+1 of a line carries cell j's rate, a non-wrapped
// edge has no face, and L is the face-weighted Laplacian along a line:
//   w  = (I - Lx/2)^-1 (I + Ly/2) f            x-sweep  (FwdX)
//   v  = (I - Ly/2)^-1 (I + Lx/2) w            y-sweep  (FwdY)
//   f' = f + (((v - f) + f*(-decay)) + src)    PDEGrid2D tick order
// For a constant rate this is Internal::Diffusion2DADI plus the tick.
//
// Every line has its own tridiagonal matrix, so the line solves are parallel
// cyclic reduction in shared memory (one CTA per line, one row per thread);
// a wrapped line of a power-of-two length reduces cyclically, any other
// wrapped line by a Sherman-Morrison split (PcrSolveSM).
//
// Gradient of loss = 1/2 |f_T - target|^2.  I - L/2 and I + L/2 are
// symmetric, so with gbar the adjoint of a step's output:
//   b2bar = (I - Ly/2)^-1 gbar;        wbar = (I + Lx/2) b2bar
//   b1bar = (I - Lx/2)^-1 wbar;        fbar = (I + Ly/2) b1bar - decay gbar
//   dsrc += gbar;   ddecay -= <gbar, f>
//   dD[owner of face] += -1/2 (p_j+1 - p_j)(q_j+1 - q_j) for the pairs
//   (b2bar, v) and (b1bar, f) on y-faces, (b2bar, w) and (b1bar, w) on x-faces
// Two kernels per backward step: BwdY applies the previous step's (I + Ly/2)
// and then this step's y-solve (both along y), BwdX the x-stencil and x-solve.
// States are recomputed segment by segment from checkpoints every k steps,
// each segment on a second stream while the one after it is differentiated.
//
// Layout: every array is row-major x*yDim + y (HAL's layout), except the
// x-kernels' own copies, which are line by line (y*xDim + x) so that an x-line
// CTA reads them contiguously: the rates DT (transposed once per call), the
// kept states w (FwdX writes them so) and the x-faces' part of dL/dD (added
// into dD once at the end).  Only the arrays passed between the sweeps (f, w
// for the y-sweep, b2bar, b1bar) keep HAL's layout and are strided for x-lines.
#include "common.cuh"
#include "adi_sweep.h"

#include <algorithm>
#include <cmath>
#include <utility>
#include <vector>

namespace halcuda
{
    namespace
    {
        constexpr int kMaxAdjLine = HAL_CUDA_ADJOINT_MAX_SIDE;

        enum LineDir : int
        {
            kDirX = 0,  // line = fixed y, positions along x (stride yDim)
            kDirY = 1   // line = fixed x, positions along y (contiguous)
        };

        struct Grid
        {
            int32_t xDim, yDim;
            int32_t wrapX, wrapY;
        };

        template <int DIR>
        __device__ __forceinline__ int64_t Idx(const Grid &g, int32_t line, int32_t pos)
        {
            return (DIR == kDirY) ? static_cast<int64_t>(line) * g.yDim + pos
                                  : static_cast<int64_t>(pos) * g.yDim + line;
        }

        template <int DIR>
        __device__ __forceinline__ int32_t LineLen(const Grid &g)
        {
            return (DIR == kDirY) ? g.yDim : g.xDim;
        }

        template <int DIR>
        __device__ __forceinline__ int32_t Lines(const Grid &g)
        {
            return (DIR == kDirY) ? g.xDim : g.yDim;
        }

        template <int DIR>
        __device__ __forceinline__ bool Wrap(const Grid &g)
        {
            return (DIR == kDirY) ? g.wrapY != 0 : g.wrapX != 0;
        }

        template <int DIR>
        __device__ __forceinline__ bool WrapCross(const Grid &g)
        {
            return (DIR == kDirY) ? g.wrapX != 0 : g.wrapY != 0;
        }

        // Face weights below (eL) and above (eR) position j of a line whose
        // rates sit in sD (one per position).
        __device__ __forceinline__ void Faces(const float *sD, int32_t j, int32_t n, bool wrap, float &eL, float &eR)
        {
            eL = (j > 0) ? sD[j - 1] : (wrap ? sD[n - 1] : 0.0f);
            eR = (j < n - 1) ? sD[j] : (wrap ? sD[n - 1] : 0.0f);
        }

        // (L u)_j along the line, with the line's u and rates in shared memory.
        __device__ __forceinline__ float LapAlong(const float *su, const float *sD, int32_t j, int32_t n, bool wrap)
        {
            float eL, eR;
            Faces(sD, j, n, wrap, eL, eR);
            const float c = su[j];
            const float lo = (j > 0) ? su[j - 1] : (wrap ? su[n - 1] : c);
            const float hi = (j < n - 1) ? su[j + 1] : (wrap ? su[0] : c);
            return eR * (hi - c) + eL * (lo - c);
        }

        // (L_cross u) at (line, j): the neighbours are lines line-1 and
        // line+1; the face (line, line+1) carries D(line, j), the face
        // (line-1, line) carries D(line-1, j).
        template <int DIR>
        __device__ __forceinline__ float LapCross(const Grid &g, const float *__restrict__ u,
                                                  const float *__restrict__ D, int32_t line, int32_t j, float c)
        {
            const int32_t nl = Lines<DIR>(g);
            const bool wrap = WrapCross<DIR>(g);
            float acc = 0.0f;
            if (line + 1 < nl || (wrap && nl > 1))
            {
                const int32_t up = (line + 1 < nl) ? line + 1 : 0;
                acc += D[Idx<DIR>(g, line, j)] * (u[Idx<DIR>(g, up, j)] - c);
            }
            if (line > 0 || (wrap && nl > 1))
            {
                const int32_t dn = (line > 0) ? line - 1 : nl - 1;
                acc += D[Idx<DIR>(g, dn, j)] * (u[Idx<DIR>(g, dn, j)] - c);
            }
            return acc;
        }

        // LapCross<kDirX> with the rates read from DT, D transposed (DT[y *
        // xDim + x] = D(x, y)): the two cross faces' rates of an x-line are then
        // contiguous along the line, like the line's own.
        __device__ __forceinline__ float LapCrossXT(const Grid &g, const float *__restrict__ u,
                                                    const float *__restrict__ DT, int32_t line, int32_t j, float c)
        {
            const int32_t nl = g.yDim;
            const bool wrap = g.wrapY != 0;
            float acc = 0.0f;
            if (line + 1 < nl || (wrap && nl > 1))
            {
                const int32_t up = (line + 1 < nl) ? line + 1 : 0;
                acc += DT[static_cast<int64_t>(line) * g.xDim + j] * (u[Idx<kDirX>(g, up, j)] - c);
            }
            if (line > 0 || (wrap && nl > 1))
            {
                const int32_t dn = (line > 0) ? line - 1 : nl - 1;
                acc += DT[static_cast<int64_t>(dn) * g.xDim + j] * (u[Idx<kDirX>(g, dn, j)] - c);
            }
            return acc;
        }

        // -1/2 (p_j+1 - p_j)(q_j+1 - q_j) for the face above position j (the
        // face owned by j), 0 if it does not exist.
        __device__ __forceinline__ float FaceGrad(const float *sp, const float *sq, int32_t j, int32_t n, bool wrap)
        {
            if (j < n - 1)
            {
                return -0.5f * (sp[j + 1] - sp[j]) * (sq[j + 1] - sq[j]);
            }
            if (wrap && n > 1)
            {
                return -0.5f * (sp[0] - sp[j]) * (sq[0] - sq[j]);
            }
            return 0.0f;
        }

        // A wrapped line whose length is not a power of two: the cyclic
        // system A x = d is split as A = T + u v^T (TdmaSolver::TDMAperiodic's
        // form, include/Hal/Pde/TdmaSolver.h:68-120: gamma = -b_0, T's
        // diagonal b_0 - gamma and b_{n-1} - a_0 c_{n-1} / gamma, u = (gamma,
        // 0, .., 0, c_{n-1}), v = (1, 0, .., 0, a_0 / gamma)); T y = d and
        // T z = u are solved together by non-wrapped parallel cyclic reduction
        // (the reductions of T are shared), then x = y - (v.y / (1 + v.z)) z.
        // sm holds 4 * blockDim.x floats, sm2 blockDim.x + 4.
        __device__ float PcrSolveSM(const float *sD, float d, int32_t j, int32_t n, float *sm, float *sm2)
        {
            float *sa = sm, *sb = sm + blockDim.x, *sc = sb + blockDim.x, *sd = sc + blockDim.x;
            float *sd2 = sm2, *sx = sm2 + blockDim.x;
            float eL0, eR0, eLn, eRn;
            Faces(sD, 0, n, true, eL0, eR0);
            Faces(sD, n - 1, n, true, eLn, eRn);
            const float a0 = -0.5f * eL0;                 // row 0's coefficient of x_{n-1}
            const float cn = -0.5f * eRn;                 // row n-1's coefficient of x_0
            const float gam = -(1.0f + 0.5f * (eL0 + eR0));  // -b_0
            float a = 0.0f, b = 1.0f, c = 0.0f, d2 = 0.0f;
            if (j < n)
            {
                float eL, eR;
                Faces(sD, j, n, true, eL, eR);
                a = (j > 0) ? -0.5f * eL : 0.0f;
                c = (j < n - 1) ? -0.5f * eR : 0.0f;
                b = 1.0f + 0.5f * (eL + eR);
                if (j == 0)
                {
                    b -= gam;
                    d2 = gam;
                }
                if (j == n - 1)
                {
                    b -= a0 * cn / gam;
                    d2 = cn;
                }
            }
            for (int32_t delta = 1; delta < n; delta <<= 1)
            {
                if (j < n)
                {
                    sa[j] = a;
                    sb[j] = b;
                    sc[j] = c;
                    sd[j] = d;
                    sd2[j] = d2;
                }
                __syncthreads();
                if (j < n)
                {
                    float al = 0.0f, bl = 1.0f, cl = 0.0f, dl = 0.0f, dl2 = 0.0f;
                    float ar = 0.0f, br = 1.0f, cr = 0.0f, dr = 0.0f, dr2 = 0.0f;
                    const int32_t il = j - delta, ir = j + delta;
                    if (il >= 0)
                    {
                        al = sa[il];
                        bl = sb[il];
                        cl = sc[il];
                        dl = sd[il];
                        dl2 = sd2[il];
                    }
                    if (ir < n)
                    {
                        ar = sa[ir];
                        br = sb[ir];
                        cr = sc[ir];
                        dr = sd[ir];
                        dr2 = sd2[ir];
                    }
                    const float alpha = -__fdividef(a, bl);
                    const float beta = -__fdividef(c, br);
                    b = b + alpha * cl + beta * ar;
                    d = d + alpha * dl + beta * dr;
                    d2 = d2 + alpha * dl2 + beta * dr2;
                    a = alpha * al;
                    c = beta * cr;
                }
                __syncthreads();
            }
            const float y = d / b, z = d2 / b;
            if (j == 0)
            {
                sx[0] = y;
                sx[2] = z;
            }
            if (j == n - 1)
            {
                sx[1] = y;
                sx[3] = z;
            }
            __syncthreads();
            const float bog = a0 / gam;
            const float fct = (sx[0] + bog * sx[1]) / (1.0f + (sx[2] + bog * sx[3]));
            return y - fct * z;
        }

        // Solves (I - L/2) x = d along the line by parallel cyclic reduction;
        // thread j holds row j (j < n); sm holds 4 * blockDim.x floats.  SMW:
        // the line wraps and its length is not a power of two (PcrSolveSM,
        // which uses blockDim.x + 4 more floats after the four line arrays);
        // a separate instantiation, so that the other line kernels keep their
        // registers (32 against 38 with both forms in one kernel, and four
        // 512-thread CTAs per SM).
        template <bool SMW>
        __device__ __forceinline__ float PcrSolve(const float *sD, float d, int32_t j, int32_t n, bool wrap, float *sm)
        {
            if constexpr (SMW)
            {
                return PcrSolveSM(sD, d, j, n, sm, sm + 8 * blockDim.x);
            }
            float *sa = sm, *sb = sm + blockDim.x, *sc = sb + blockDim.x, *sd = sc + blockDim.x;
            float a = 0.0f, b = 1.0f, c = 0.0f;
            if (j < n)
            {
                float eL, eR;
                Faces(sD, j, n, wrap, eL, eR);
                a = -0.5f * eL;
                c = -0.5f * eR;
                b = 1.0f + 0.5f * (eL + eR);
            }
            for (int32_t delta = 1; delta < n; delta <<= 1)
            {
                if (j < n)
                {
                    sa[j] = a;
                    sb[j] = b;
                    sc[j] = c;
                    sd[j] = d;
                }
                __syncthreads();
                if (j < n)
                {
                    float al = 0.0f, bl = 1.0f, cl = 0.0f, dl = 0.0f;
                    float ar = 0.0f, br = 1.0f, cr = 0.0f, dr = 0.0f;
                    int32_t il = j - delta, ir = j + delta;
                    if (wrap)
                    {
                        il = (il < 0) ? il + n : il;
                        ir = (ir >= n) ? ir - n : ir;
                    }
                    if (il >= 0)
                    {
                        al = sa[il];
                        bl = sb[il];
                        cl = sc[il];
                        dl = sd[il];
                    }
                    if (ir < n)
                    {
                        ar = sa[ir];
                        br = sb[ir];
                        cr = sc[ir];
                        dr = sd[ir];
                    }
                    // fast reciprocal division (about 2 ulp): the rows are
                    // diagonally dominant, so the reduction stays well
                    // conditioned
                    const float alpha = -__fdividef(a, bl);
                    const float gamma = -__fdividef(c, br);
                    b = b + alpha * cl + gamma * ar;
                    d = d + alpha * dl + gamma * dr;
                    a = alpha * al;
                    c = gamma * cr;
                }
                __syncthreads();
            }
            // non-wrapped: every coupling left the line; wrapped: the last
            // step coupled each row to itself
            return wrap ? d / (a + b + c) : d / b;
        }

        __device__ __forceinline__ double BlockSum(double v, double *sred)
        {
            for (int o = 16; o > 0; o >>= 1)
            {
                v += __shfl_down_sync(0xffffffffu, v, o);
            }
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
            __syncthreads();
            if (lane == 0)
            {
                sred[warp] = v;
            }
            __syncthreads();
            double t = 0.0;
            if (threadIdx.x == 0)
            {
                for (int k = 0; k < static_cast<int>((blockDim.x + 31) / 32); k++)
                {
                    t += sred[k];
                }
            }
            return t;
        }

        // A wrapped line of length n that is not a power of two: its solve is
        // the Sherman-Morrison form (the line kernels' SMW instantiation).
        __host__ __device__ constexpr bool SmLine(int32_t n, bool wrap)
        {
            return wrap && n > 2 && (n & (n - 1)) != 0;
        }

        // Shared memory of the line kernels: 4 PCR arrays + 4 line arrays,
        // and for an SmLine the second right-hand side and the broadcast
        // values of PcrSolveSM.
        __host__ __device__ constexpr size_t LineSmemFloats(int threads, int32_t n, bool wrap)
        {
            return SmLine(n, wrap) ? 9 * static_cast<size_t>(threads) + 4 : 8 * static_cast<size_t>(threads);
        }

        // x-sweep: w = (I - Lx/2)^-1 (I + Ly/2) f, one CTA per line y, in
        // residual form: w = f + (I - Lx/2)^-1 (Lx + Ly) f / 2, so that the
        // solve's rounding scales with the step's change, not the field.  The
        // rates come from DT (D transposed), contiguous along the line.  w is
        // written in HAL's layout for the y-sweep, and, when wB is set, also
        // line by line (wB[y * xDim + x]) as the state the backward x-kernel
        // reads along the same lines.
        template <bool SMW>
        __global__ void FwdX(Grid g, const float *__restrict__ f, const float *__restrict__ DT, float *__restrict__ w,
                             float *__restrict__ wB)
        {
            extern __shared__ float sm[];
            float *sD = sm + 4 * blockDim.x;
            float *su = sD + blockDim.x;
            const int32_t line = blockIdx.x;
            const int32_t n = g.xDim;
            const int32_t j = threadIdx.x;
            float c = 0.0f, lap = 0.0f;
            if (j < n)
            {
                const int64_t i = Idx<kDirX>(g, line, j);
                sD[j] = DT[static_cast<int64_t>(line) * n + j];
                c = f[i];
                su[j] = c;
                lap = LapCrossXT(g, f, DT, line, j, c);
            }
            __syncthreads();
            if (j < n)
            {
                lap += LapAlong(su, sD, j, n, g.wrapX != 0);
            }
            const float e = PcrSolve<SMW>(sD, 0.5f * lap, j, n, g.wrapX != 0, sm);
            if (j < n)
            {
                w[Idx<kDirX>(g, line, j)] = c + e;
                if (wB != nullptr)
                {
                    wB[static_cast<int64_t>(line) * n + j] = c + e;
                }
            }
        }

        // y-sweep and commit: v = (I - Ly/2)^-1 (I + Lx/2) w,
        // f' = f + (((v - f) + f*(-decay)) + src); v is kept when vOut != null.
        template <bool SMW>
        __global__ void FwdY(Grid g, const float *__restrict__ w, const float *__restrict__ f,
                             const float *__restrict__ D, const float *__restrict__ src, float negDecay,
                             float *__restrict__ fOut, float *__restrict__ vOut)
        {
            extern __shared__ float sm[];
            float *sD = sm + 4 * blockDim.x;
            float *su = sD + blockDim.x;
            const int32_t line = blockIdx.x;
            const int32_t n = g.yDim;
            const int32_t j = threadIdx.x;
            float c = 0.0f, lap = 0.0f;
            if (j < n)
            {
                const int64_t i = Idx<kDirY>(g, line, j);
                sD[j] = D[i];
                c = w[i];
                su[j] = c;
                lap = LapCross<kDirY>(g, w, D, line, j, c);
            }
            __syncthreads();
            if (j < n)
            {
                lap += LapAlong(su, sD, j, n, g.wrapY != 0);
            }
            // residual form: v = w + (I - Ly/2)^-1 (Lx + Ly) w / 2
            const float e = PcrSolve<SMW>(sD, 0.5f * lap, j, n, g.wrapY != 0, sm);
            if (j < n)
            {
                const int64_t i = Idx<kDirY>(g, line, j);
                const float f0 = f[i];
                // v - f = (w - f) + e: both small, so the commit keeps the
                // field's precision
                float delta = (c - f0) + e;
                delta = delta + f0 * negDecay;
                if (src != nullptr)
                {
                    delta = delta + src[i];
                }
                fOut[i] = f0 + delta;
                if (vOut != nullptr)
                {
                    vOut[i] = c + e;
                }
            }
        }

        // loss += 1/2 (f - target)^2; gbar = f - target.
        __global__ void LossGrad(int64_t n, const float *__restrict__ f, const float *__restrict__ target,
                                 float *__restrict__ gbar, double *__restrict__ loss)
        {
            __shared__ double sred[32];
            double acc = 0.0;
            for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
                 i += static_cast<int64_t>(gridDim.x) * blockDim.x)
            {
                const float r = f[i] - target[i];
                if (gbar != nullptr)
                {
                    gbar[i] = r;
                }
                acc += 0.5 * static_cast<double>(r) * static_cast<double>(r);
            }
            const double t = BlockSum(acc, sred);
            if (threadIdx.x == 0)
            {
                atomicAdd(loss, t);
            }
        }

        enum BwdYMode : int
        {
            kBwdFirst = 0,  // gbar given (the last step's output adjoint)
            kBwdNext = 1,   // gbar = (I + Ly/2) b1bar - decay gbarPrev
            kBwdTail = 2    // the y-stencil part of kBwdNext only (after step 0)
        };

        // Backward along y for step t: [gbar from step t+1] then the y-solve.
        template <bool SMW>
        __global__ void BwdY(Grid g, int mode, const float *__restrict__ D, float decay,
                             const float *__restrict__ b1bar,     // step t+1's x-solve adjoint (kBwdNext/Tail)
                             const float *__restrict__ gPrev,     // adjoint of f_t+2 (kBwdNext/Tail), or gbar (kBwdFirst)
                             const float *__restrict__ fNext,     // f_t+1 (kBwdNext/Tail)
                             const float *__restrict__ fT,        // f_t (input of step t)
                             const float *__restrict__ vT,        // v_t
                             float *__restrict__ gOut,            // adjoint of f_t+1 (gbar of step t)
                             float *__restrict__ b2bar, float *__restrict__ dD, float *__restrict__ dS,
                             double *__restrict__ dDecay)
        {
            extern __shared__ float sm[];
            float *sD = sm + 4 * blockDim.x;
            float *sp = sD + blockDim.x;
            float *sq = sp + blockDim.x;
            float *sr = sq + blockDim.x;
            __shared__ double sred[32];
            const int32_t line = blockIdx.x;
            const int32_t n = g.yDim;
            const bool wrap = g.wrapY != 0;
            const int32_t j = threadIdx.x;
            const int64_t i = (j < n) ? Idx<kDirY>(g, line, j) : 0;
            float gbar = 0.0f, dDacc = 0.0f;
            if (j < n)
            {
                sD[j] = D[i];
                if (mode == kBwdFirst)
                {
                    gbar = gPrev[i];
                }
                else
                {
                    sp[j] = b1bar[i];
                    sq[j] = fNext[i];
                }
            }
            __syncthreads();
            if (mode != kBwdFirst)
            {
                if (j < n)
                {
                    gbar = (sp[j] + 0.5f * LapAlong(sp, sD, j, n, wrap)) - decay * gPrev[i];
                    dDacc += FaceGrad(sp, sq, j, n, wrap);
                }
                if (mode == kBwdTail)
                {
                    if (j < n)
                    {
                        dD[i] += dDacc;
                    }
                    return;
                }
            }
            double kacc = 0.0;
            if (j < n)
            {
                dS[i] += gbar;
                kacc = -static_cast<double>(gbar) * static_cast<double>(fT[i]);
                gOut[i] = gbar;
            }
            const double ksum = BlockSum(kacc, sred);
            if (threadIdx.x == 0)
            {
                atomicAdd(dDecay, ksum);
            }
            // residual form: b2bar = gbar + (I - Ly/2)^-1 (Ly gbar) / 2
            if (j < n)
            {
                sq[j] = gbar;
            }
            __syncthreads();
            const float lapg = (j < n) ? LapAlong(sq, sD, j, n, wrap) : 0.0f;
            const float x = gbar + PcrSolve<SMW>(sD, 0.5f * lapg, j, n, wrap, sm);
            if (j < n)
            {
                sp[j] = x;
                sr[j] = vT[i];
            }
            __syncthreads();
            if (j < n)
            {
                dDacc += FaceGrad(sp, sr, j, n, wrap);
                b2bar[i] = x;
                dD[i] += dDacc;
            }
        }

        // Backward along x for step t: wbar = (I + Lx/2) b2bar, b1bar = (I - Lx/2)^-1 wbar.
        // The rates DT, the state wB and the x-face gradient dDT are all
        // line by line (y * xDim + x), contiguous along the CTA's line; only
        // b2bar and b1bar, which the y-kernels read and write, are strided.
        template <bool SMW>
        __global__ void BwdX(Grid g, const float *__restrict__ DT, const float *__restrict__ b2bar,
                             const float *__restrict__ wB, float *__restrict__ b1bar, float *__restrict__ dDT)
        {
            extern __shared__ float sm[];
            float *sD = sm + 4 * blockDim.x;
            float *sp = sD + blockDim.x;
            float *sw = sp + blockDim.x;
            const int32_t line = blockIdx.x;
            const int32_t n = g.xDim;
            const bool wrap = g.wrapX != 0;
            const int32_t j = threadIdx.x;
            const int64_t i = (j < n) ? Idx<kDirX>(g, line, j) : 0;
            const int64_t iB = static_cast<int64_t>(line) * n + j;
            if (j < n)
            {
                sD[j] = DT[iB];
                sp[j] = b2bar[i];
                sw[j] = wB[iB];
            }
            __syncthreads();
            float wbar = 0.0f, dDacc = 0.0f, lapb = 0.0f;
            if (j < n)
            {
                lapb = LapAlong(sp, sD, j, n, wrap);
                wbar = sp[j] + 0.5f * lapb;
                dDacc = FaceGrad(sp, sw, j, n, wrap);
            }
            // residual form: b1bar = wbar + (I - Lx/2)^-1 (Lx wbar) / 2, with
            // Lx wbar = Lx b2bar + Lx (Lx b2bar) / 2
            float *sl = sw + blockDim.x;
            if (j < n)
            {
                sl[j] = lapb;
            }
            __syncthreads();
            const float lapw = (j < n) ? lapb + 0.5f * LapAlong(sl, sD, j, n, wrap) : 0.0f;
            __syncthreads();
            const float x = wbar + PcrSolve<SMW>(sD, 0.5f * lapw, j, n, wrap, sm);
            if (j < n)
            {
                sp[j] = x;
            }
            __syncthreads();
            if (j < n)
            {
                dDacc += FaceGrad(sp, sw, j, n, wrap);
                b1bar[i] = x;
                dDT[iB] += dDacc;
            }
        }

        // dD(x, y) += dDT[y * xDim + x]: the x-faces' gradient, accumulated
        // line by line, added into HAL's layout through a 32 x 32 tile.
        __global__ void AddTransposed(float *__restrict__ dD, const float *__restrict__ dDT, int32_t xDim,
                                      int32_t yDim)
        {
            __shared__ float tile[32][33];
            const int32_t x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
            for (int32_t r = threadIdx.y; r < 32; r += blockDim.y)
            {
                const int32_t y = y0 + r, x = x0 + threadIdx.x;
                if (y < yDim && x < xDim)
                {
                    tile[r][threadIdx.x] = dDT[static_cast<int64_t>(y) * xDim + x];
                }
            }
            __syncthreads();
            for (int32_t r = threadIdx.y; r < 32; r += blockDim.y)
            {
                const int32_t x = x0 + r, y = y0 + threadIdx.x;
                if (x < xDim && y < yDim)
                {
                    dD[static_cast<int64_t>(x) * yDim + y] += tile[threadIdx.x][r];
                }
            }
        }
    }

    struct Adjoint
    {
        int device = 0;
        StreamSlot stream;
        Grid g{};
        int64_t n = 0;
        int32_t steps = 0, every = 1;
        bool keepAll = false;               // checkpoint interval 0: every state kept, nothing recomputed
        bool hasProblem = false;
        DevBuf<float> f0, target, D, src;
        DevBuf<float> ckpt;                 // checkpoints: one field every `every` steps
        DevBuf<float> segF[2], segW[2], segV[2];  // states of a segment, double-buffered
        StreamSlot recomputeStream;         // recomputes segment s-1 while segment s is differentiated
        DevBuf<float> work[2];              // forward ping-pong
        DevBuf<float> gA, gB, b1, b2, dD, dS;
        // line-by-line (y * xDim + x) copies for the x-kernels: the rates,
        // the x-faces' part of dL/dD, and the x-sweep's w in HAL's layout for
        // the y-sweep (scratch: the forward on the main stream and the
        // recomputations on the second one never run at the same time)
        DevBuf<float> DT, dDT, wA;
        DevBuf<double> acc;                 // [0] loss, [1] d loss / d decay
        float msForward = 0.0f, msGradient = 0.0f;

        int32_t Segments() const
        {
            return (steps + every - 1) / every;
        }

        int Init(int32_t xDim, int32_t yDim, int32_t wrapX, int32_t wrapY)
        {
            device = CurrentDevice();
            HAL_TRY(CudaStatus(cudaSetDevice(device), "cudaSetDevice"));
            // the backward (and the forward) on the highest-priority stream,
            // the overlapped recomputation on the lowest: recompute CTAs take
            // the SMs the critical path leaves free
            int least = 0, greatest = 0;
            HAL_TRY(CudaStatus(cudaDeviceGetStreamPriorityRange(&least, &greatest), "cudaDeviceGetStreamPriorityRange"));
            HAL_TRY(stream.Create("cudaStreamCreate", greatest));
            HAL_TRY(recomputeStream.Create("cudaStreamCreate", least));
            g.xDim = xDim;
            g.yDim = yDim;
            g.wrapX = wrapX != 0;
            g.wrapY = wrapY != 0;
            n = static_cast<int64_t>(xDim) * yDim;
            const size_t m = static_cast<size_t>(n);
            HAL_TRY(f0.Alloc(m, "cudaMalloc(adjoint)"));
            HAL_TRY(target.Alloc(m, "cudaMalloc(adjoint)"));
            HAL_TRY(D.Alloc(m, "cudaMalloc(adjoint)"));
            HAL_TRY(src.Alloc(m, "cudaMalloc(adjoint)"));
            HAL_TRY(work[0].Alloc(m, "cudaMalloc(adjoint)"));
            HAL_TRY(work[1].Alloc(m, "cudaMalloc(adjoint)"));
            HAL_TRY(gA.Alloc(m, "cudaMalloc(adjoint)"));
            HAL_TRY(gB.Alloc(m, "cudaMalloc(adjoint)"));
            HAL_TRY(b1.Alloc(m, "cudaMalloc(adjoint)"));
            HAL_TRY(b2.Alloc(m, "cudaMalloc(adjoint)"));
            HAL_TRY(dD.Alloc(m, "cudaMalloc(adjoint)"));
            HAL_TRY(DT.Alloc(m, "cudaMalloc(adjoint)"));
            HAL_TRY(dDT.Alloc(m, "cudaMalloc(adjoint)"));
            HAL_TRY(wA.Alloc(m, "cudaMalloc(adjoint)"));
            HAL_TRY(dS.Alloc(m, "cudaMalloc(adjoint)"));
            HAL_TRY(acc.Alloc(2, "cudaMalloc(adjoint)"));
            return HAL_CUDA_OK;
        }

        static int Threads(int32_t len)
        {
            return (len + 31) & ~31;
        }

        // One forward step fIn -> fOut; the step's w is kept line by line in
        // wKeep and its v in vOut when they are set.
        int LaunchFwd(const float *fIn, float *fOut, float *wKeep, float *vOut, const float *srcp, float negDecay,
                      cudaStream_t s)
        {
            const int tx = Threads(g.xDim), ty = Threads(g.yDim);
            const auto fwdX = SmLine(g.xDim, g.wrapX != 0) ? FwdX<true> : FwdX<false>;
            const auto fwdY = SmLine(g.yDim, g.wrapY != 0) ? FwdY<true> : FwdY<false>;
            fwdX<<<g.yDim, tx, LineSmemFloats(tx, g.xDim, g.wrapX != 0) * sizeof(float), s>>>(g, fIn, DT.p, wA.p, wKeep);
            fwdY<<<g.xDim, ty, LineSmemFloats(ty, g.yDim, g.wrapY != 0) * sizeof(float), s>>>(g, wA.p, fIn, D.p,
                                                                                               srcp, negDecay, fOut,
                                                                         vOut);
            CountLaunch(2);
            return LaunchStatus("adjoint forward step");
        }

        int Upload(const float *hD, const float *hSrc, bool &useSrc, cudaStream_t s)
        {
            const size_t bytes = static_cast<size_t>(n) * sizeof(float);
            HAL_TRY(CudaStatus(cudaMemcpyAsync(D.p, hD, bytes, cudaMemcpyHostToDevice, s), "cudaMemcpy(D)"));
            HAL_TRY(LaunchTranspose(D.p, DT.p, g.xDim, g.yDim, s));
            useSrc = (hSrc != nullptr);
            if (useSrc)
            {
                HAL_TRY(CudaStatus(cudaMemcpyAsync(src.p, hSrc, bytes, cudaMemcpyHostToDevice, s), "cudaMemcpy(src)"));
            }
            return HAL_CUDA_OK;
        }

        // `steps` forward steps from f0; checkpoints stored when ck != null.
        // Returns the buffer holding f_T.
        const float *Forward(const float *srcp, float negDecay, float *ck, cudaStream_t s, int &rc)
        {
            const size_t bytes = static_cast<size_t>(n) * sizeof(float);
            rc = CudaStatus(cudaMemcpyAsync(work[0].p, f0.p, bytes, cudaMemcpyDeviceToDevice, s), "cudaMemcpy(f0)");
            int c = 0;
            for (int32_t t = 0; t < steps && rc == HAL_CUDA_OK; t++)
            {
                if (ck != nullptr && t % every == 0)
                {
                    rc = CudaStatus(cudaMemcpyAsync(ck + static_cast<size_t>(t / every) * n, work[c].p, bytes,
                                                    cudaMemcpyDeviceToDevice, s), "cudaMemcpy(checkpoint)");
                }
                if (rc == HAL_CUDA_OK)
                {
                    rc = LaunchFwd(work[c].p, work[c ^ 1].p, nullptr, nullptr, srcp, negDecay, s);
                }
                c ^= 1;
            }
            return work[c].p;
        }

        int LaunchLoss(const float *fT, float *gbar, cudaStream_t s)
        {
            const int T = 256;
            const int blocks = static_cast<int>(std::min<int64_t>((n + T - 1) / T, 1024));
            LossGrad<<<blocks, T, 0, s>>>(n, fT, target.p, gbar, acc.p);
            CountLaunch();
            return LaunchStatus("adjoint loss");
        }

        int RunForward(const float *hD, double decay, const float *hSrc, double *loss, float *hFT)
        {
            cudaStream_t s = stream.Get();
            bool useSrc = false;
            HAL_TRY(Upload(hD, hSrc, useSrc, s));
            HAL_TRY(CudaStatus(cudaMemsetAsync(acc.p, 0, 2 * sizeof(double), s), "cudaMemset(acc)"));
            cudaEvent_t e0, e1;
            HAL_TRY(CudaStatus(cudaEventCreate(&e0), "cudaEventCreate"));
            HAL_TRY(CudaStatus(cudaEventCreate(&e1), "cudaEventCreate"));
            cudaEventRecord(e0, s);
            int rc = HAL_CUDA_OK;
            const float *fT = Forward(useSrc ? src.p : nullptr, static_cast<float>(-decay), nullptr, s, rc);
            if (rc == HAL_CUDA_OK)
            {
                rc = LaunchLoss(fT, nullptr, s);
            }
            cudaEventRecord(e1, s);
            double h[2] = {0, 0};
            if (rc == HAL_CUDA_OK)
            {
                rc = CudaStatus(cudaMemcpyAsync(h, acc.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s),
                                "cudaMemcpy(loss)");
            }
            if (rc == HAL_CUDA_OK && hFT != nullptr)
            {
                rc = CudaStatus(cudaMemcpyAsync(hFT, fT, static_cast<size_t>(n) * sizeof(float), cudaMemcpyDeviceToHost,
                                                s), "cudaMemcpy(f_T)");
            }
            if (rc == HAL_CUDA_OK)
            {
                rc = CudaStatus(cudaStreamSynchronize(s), "adjoint forward");
            }
            if (rc == HAL_CUDA_OK)
            {
                cudaEventElapsedTime(&msForward, e0, e1);
                *loss = h[0];
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return rc;
        }

        int RunGradient(const float *hD, double decay, const float *hSrc, double *loss, float *hgD, double *hgK,
                        float *hgS)
        {
            cudaStream_t s = stream.Get();
            bool useSrc = false;
            HAL_TRY(Upload(hD, hSrc, useSrc, s));
            const size_t bytes = static_cast<size_t>(n) * sizeof(float);
            const float *srcp = useSrc ? src.p : nullptr;
            const float negDecay = static_cast<float>(-decay);
            HAL_TRY(CudaStatus(cudaMemsetAsync(acc.p, 0, 2 * sizeof(double), s), "cudaMemset(acc)"));
            HAL_TRY(CudaStatus(cudaMemsetAsync(dD.p, 0, bytes, s), "cudaMemset(dD)"));
            HAL_TRY(CudaStatus(cudaMemsetAsync(dDT.p, 0, bytes, s), "cudaMemset(dD)"));
            HAL_TRY(CudaStatus(cudaMemsetAsync(dS.p, 0, bytes, s), "cudaMemset(dS)"));
            cudaEvent_t e0, e1;
            HAL_TRY(CudaStatus(cudaEventCreate(&e0), "cudaEventCreate"));
            HAL_TRY(CudaStatus(cudaEventCreate(&e1), "cudaEventCreate"));
            cudaEventRecord(e0, s);
            int rc = HAL_CUDA_OK;
            float *gCur = gA.p, *gNext = gB.p;  // gCur: adjoint of the latest output handled
            const int tx = Threads(g.xDim), ty = Threads(g.yDim);
            const size_t smx = LineSmemFloats(tx, g.xDim, g.wrapX != 0) * sizeof(float);
            const size_t smy = LineSmemFloats(ty, g.yDim, g.wrapY != 0) * sizeof(float);
            const auto bwdX = SmLine(g.xDim, g.wrapX != 0) ? BwdX<true> : BwdX<false>;
            const auto bwdY = SmLine(g.yDim, g.wrapY != 0) ? BwdY<true> : BwdY<false>;
            bool first = true;
            // states f_t0..f_t1, w and v of one segment into buffer b, from
            // the field at t0, on stream rs
            auto recompute = [&](int b, const float *from, int32_t t0, int32_t t1, cudaStream_t rs) {
                int r = CudaStatus(cudaMemcpyAsync(segF[b].p, from, bytes, cudaMemcpyDeviceToDevice, rs),
                                   "cudaMemcpy(segment)");
                for (int32_t t = t0; t < t1 && r == HAL_CUDA_OK; t++)
                {
                    const size_t k = static_cast<size_t>(t - t0);
                    r = LaunchFwd(segF[b].p + k * n, segF[b].p + (k + 1) * n, segW[b].p + k * n, segV[b].p + k * n,
                                  srcp, negDecay, rs);
                }
                return r;
            };
            // reverse steps t1-1 .. t0 over the states in buffer b
            auto backward = [&](int b, int32_t t0, int32_t t1) {
                int r = HAL_CUDA_OK;
                for (int32_t t = t1 - 1; t >= t0 && r == HAL_CUDA_OK; t--)
                {
                    const size_t k = static_cast<size_t>(t - t0);
                    const float *fNext = segF[b].p + (k + 1) * n;
                    bwdY<<<g.xDim, ty, smy, s>>>(g, first ? kBwdFirst : kBwdNext, D.p, static_cast<float>(decay),
                                                 b1.p, gCur, fNext, segF[b].p + k * n, segV[b].p + k * n, gNext,
                                                 b2.p, dD.p, dS.p, acc.p + 1);
                    bwdX<<<g.yDim, tx, smx, s>>>(g, DT.p, b2.p, segW[b].p + k * n, b1.p, dDT.p);
                    CountLaunch(2);
                    r = LaunchStatus("adjoint backward step");
                    std::swap(gCur, gNext);
                    first = false;
                }
                return r;
            };
            int lastBuf = 0;  // buffer of segment 0, read by the tail step
            if (keepAll)
            {
                // every state of the run is kept: one forward pass, no recomputation
                rc = recompute(0, f0.p, 0, steps, s);
                if (rc == HAL_CUDA_OK)
                {
                    rc = LaunchLoss(segF[0].p + static_cast<size_t>(steps) * n, gCur, s);
                }
                if (rc == HAL_CUDA_OK)
                {
                    rc = backward(0, 0, steps);
                }
            }
            else
            {
                // Segments are differentiated last to first.  Segment s-1 is
                // recomputed from its checkpoint on a second stream into the
                // other buffer while segment s is differentiated; events order
                // each buffer's writer (recompute) and reader (backward).
                cudaStream_t rs = recomputeStream.Get();
                cudaEvent_t ready = nullptr, recDone[2] = {nullptr, nullptr}, bwdDone[2] = {nullptr, nullptr};
                for (cudaEvent_t *e : {&ready, &recDone[0], &recDone[1], &bwdDone[0], &bwdDone[1]})
                {
                    if (rc == HAL_CUDA_OK)
                    {
                        rc = CudaStatus(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "cudaEventCreate");
                    }
                }
                // The forward pass keeps checkpoints, and writes the states of
                // the last two segments (one per buffer) as it goes, so the
                // backward starts without waiting for a recomputation.
                const int32_t S = Segments();
                const int32_t firstKept = std::max(S - 2, 0);
                const float *fT = nullptr;
                if (rc == HAL_CUDA_OK)
                {
                    rc = CudaStatus(cudaMemcpyAsync(work[0].p, f0.p, bytes, cudaMemcpyDeviceToDevice, s),
                                    "cudaMemcpy(f0)");
                }
                const float *fCur = work[0].p;
                int c = 0;
                for (int32_t t = 0; t < steps && rc == HAL_CUDA_OK; t++)
                {
                    const int32_t seg = t / every;
                    if (t % every == 0)
                    {
                        rc = CudaStatus(cudaMemcpyAsync(ckpt.p + static_cast<size_t>(seg) * n, fCur, bytes,
                                                        cudaMemcpyDeviceToDevice, s), "cudaMemcpy(checkpoint)");
                        if (rc == HAL_CUDA_OK && seg >= firstKept)
                        {
                            rc = CudaStatus(cudaMemcpyAsync(segF[seg & 1].p, fCur, bytes, cudaMemcpyDeviceToDevice, s),
                                            "cudaMemcpy(segment)");
                        }
                    }
                    if (rc != HAL_CUDA_OK)
                    {
                        break;
                    }
                    if (seg >= firstKept)
                    {
                        const int b = seg & 1;
                        const size_t k = static_cast<size_t>(t - seg * every);
                        float *fOut = segF[b].p + (k + 1) * n;
                        rc = LaunchFwd(fCur, fOut, segW[b].p + k * n, segV[b].p + k * n, srcp, negDecay, s);
                        fCur = fOut;
                    }
                    else
                    {
                        rc = LaunchFwd(fCur, work[c ^ 1].p, nullptr, nullptr, srcp, negDecay, s);
                        c ^= 1;
                        fCur = work[c].p;
                    }
                }
                fT = fCur;
                if (rc == HAL_CUDA_OK)
                {
                    rc = LaunchLoss(fT, gCur, s);
                }
                auto enqueueRecompute = [&](int32_t seg) {
                    if (seg >= firstKept)
                    {
                        return static_cast<int>(HAL_CUDA_OK);  // written by the forward pass
                    }
                    const int b = seg & 1;
                    const int32_t t0 = seg * every;
                    // the buffer's previous reader is the backward of segment seg+2
                    int r = CudaStatus(cudaStreamWaitEvent(rs, bwdDone[b], 0), "cudaStreamWaitEvent");
                    if (r == HAL_CUDA_OK)
                    {
                        r = recompute(b, ckpt.p + static_cast<size_t>(seg) * n, t0, std::min(steps, t0 + every), rs);
                    }
                    if (r == HAL_CUDA_OK)
                    {
                        r = CudaStatus(cudaEventRecord(recDone[b], rs), "cudaEventRecord");
                    }
                    return r;
                };
                if (rc == HAL_CUDA_OK)
                {
                    // the checkpoints are written by the forward pass on s
                    rc = CudaStatus(cudaEventRecord(ready, s), "cudaEventRecord");
                }
                if (rc == HAL_CUDA_OK)
                {
                    rc = CudaStatus(cudaStreamWaitEvent(rs, ready, 0), "cudaStreamWaitEvent");
                }
                if (rc == HAL_CUDA_OK && S > 0)
                {
                    rc = enqueueRecompute(S - 1);
                }
                for (int32_t seg = S - 1; seg >= 0 && rc == HAL_CUDA_OK; seg--)
                {
                    if (seg > 0)
                    {
                        rc = enqueueRecompute(seg - 1);
                    }
                    const int b = seg & 1;
                    const int32_t t0 = seg * every;
                    if (rc == HAL_CUDA_OK)
                    {
                        rc = CudaStatus(cudaStreamWaitEvent(s, recDone[b], 0), "cudaStreamWaitEvent");
                    }
                    if (rc == HAL_CUDA_OK)
                    {
                        rc = backward(b, t0, std::min(steps, t0 + every));
                    }
                    if (rc == HAL_CUDA_OK)
                    {
                        rc = CudaStatus(cudaEventRecord(bwdDone[b], s), "cudaEventRecord");
                    }
                }
                // s now follows every recompute (each backward waited on its
                // own); an early failure still leaves rs to be drained
                if (rc != HAL_CUDA_OK)
                {
                    cudaStreamSynchronize(rs);
                }
                for (cudaEvent_t e : {ready, recDone[0], recDone[1], bwdDone[0], bwdDone[1]})
                {
                    if (e != nullptr)
                    {
                        cudaEventDestroy(e);
                    }
                }
            }
            if (rc == HAL_CUDA_OK && steps > 0)
            {
                // the y-stencil part of step 0's (I + Ly/2) b1bar: its D terms
                bwdY<<<g.xDim, ty, smy, s>>>(g, kBwdTail, D.p, static_cast<float>(decay), b1.p, gCur,
                                             segF[lastBuf].p, segF[lastBuf].p, segV[lastBuf].p, gNext, b2.p, dD.p,
                                             dS.p, acc.p + 1);
                CountLaunch();
                rc = LaunchStatus("adjoint backward tail");
            }
            if (rc == HAL_CUDA_OK)
            {
                // the x-faces' part of dL/dD, accumulated line by line
                AddTransposed<<<dim3((g.xDim + 31) / 32, (g.yDim + 31) / 32), dim3(32, 8), 0, s>>>(dD.p, dDT.p,
                                                                                               g.xDim, g.yDim);
                CountLaunch();
                rc = LaunchStatus("adjoint dD");
            }
            cudaEventRecord(e1, s);
            double h[2] = {0, 0};
            if (rc == HAL_CUDA_OK)
            {
                rc = CudaStatus(cudaMemcpyAsync(h, acc.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, s),
                                "cudaMemcpy(loss)");
            }
            if (rc == HAL_CUDA_OK && hgD != nullptr)
            {
                rc = CudaStatus(cudaMemcpyAsync(hgD, dD.p, bytes, cudaMemcpyDeviceToHost, s), "cudaMemcpy(dD)");
            }
            if (rc == HAL_CUDA_OK && hgS != nullptr)
            {
                rc = CudaStatus(cudaMemcpyAsync(hgS, dS.p, bytes, cudaMemcpyDeviceToHost, s), "cudaMemcpy(dS)");
            }
            if (rc == HAL_CUDA_OK)
            {
                rc = CudaStatus(cudaStreamSynchronize(s), "adjoint gradient");
            }
            if (rc == HAL_CUDA_OK)
            {
                cudaEventElapsedTime(&msGradient, e0, e1);
                *loss = h[0];
                if (hgK != nullptr)
                {
                    *hgK = h[1];
                }
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return rc;
        }
    };
}

using halcuda::Adjoint;

struct hal_cuda_adjoint : public Adjoint
{
};

extern "C" int hal_cuda_adjoint_create(int32_t xDim, int32_t yDim, int32_t wrapX, int32_t wrapY,
                                       hal_cuda_adjoint **out)
{
    HAL_REQUIRE(out != nullptr, "hal_cuda_adjoint_create: out is NULL");
    *out = nullptr;
    HAL_REQUIRE(xDim >= 1 && yDim >= 1 && xDim <= halcuda::kMaxAdjLine && yDim <= halcuda::kMaxAdjLine,
                "hal_cuda_adjoint_create: grid %d x %d, sides must be in [1, %d]", xDim, yDim, halcuda::kMaxAdjLine);
    hal_cuda_adjoint *h = new (std::nothrow) hal_cuda_adjoint();
    if (h == nullptr)
    {
        halcuda::SetError("hal_cuda_adjoint_create: out of host memory");
        return HAL_CUDA_ENOMEM;
    }
    int rc = h->Init(xDim, yDim, wrapX, wrapY);
    if (rc != HAL_CUDA_OK)
    {
        delete h;
        return rc;
    }
    *out = h;
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_adjoint_destroy(hal_cuda_adjoint *h)
{
    if (h != nullptr)
    {
        cudaSetDevice(h->device);
        cudaStreamSynchronize(h->stream.Get());
        cudaStreamSynchronize(h->recomputeStream.Get());
        delete h;
    }
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_adjoint_set_problem(hal_cuda_adjoint *h, const float *f0, const float *target, int64_t len,
                                            int32_t steps, int32_t checkpointEvery)
{
    HAL_REQUIRE(h != nullptr && f0 != nullptr && target != nullptr, "hal_cuda_adjoint_set_problem: NULL argument");
    HAL_REQUIRE(len == h->n, "hal_cuda_adjoint_set_problem: length %lld, grid holds %lld cells",
                static_cast<long long>(len), static_cast<long long>(h->n));
    HAL_REQUIRE(steps >= 0, "hal_cuda_adjoint_set_problem: negative step count");
    HAL_REQUIRE(checkpointEvery >= 0, "hal_cuda_adjoint_set_problem: negative checkpoint interval");
    using namespace halcuda;
    HAL_TRY(CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    const size_t m = static_cast<size_t>(h->n);
    h->steps = steps;
    h->keepAll = (checkpointEvery == 0);
    h->every = h->keepAll ? std::max(steps, 1) : std::min(checkpointEvery, std::max(steps, 1));
    HAL_TRY(h->ckpt.Alloc(m * static_cast<size_t>(std::max(h->Segments(), 1)), "cudaMalloc(checkpoints)"));
    // one segment buffer when every state is kept or there is one segment,
    // two (recompute of one overlapping the backward of the other) otherwise
    const int nBuf = (h->keepAll || h->Segments() <= 1) ? 1 : 2;
    for (int b = 0; b < 2; b++)
    {
        if (b < nBuf)
        {
            HAL_TRY(h->segF[b].Alloc(m * static_cast<size_t>(h->every + 1), "cudaMalloc(segment)"));
            HAL_TRY(h->segW[b].Alloc(m * static_cast<size_t>(h->every), "cudaMalloc(segment)"));
            HAL_TRY(h->segV[b].Alloc(m * static_cast<size_t>(h->every), "cudaMalloc(segment)"));
        }
        else
        {
            h->segF[b].Free();
            h->segW[b].Free();
            h->segV[b].Free();
        }
    }
    cudaStream_t s = h->stream.Get();
    HAL_TRY(CudaStatus(cudaMemcpyAsync(h->f0.p, f0, m * sizeof(float), cudaMemcpyHostToDevice, s), "cudaMemcpy(f0)"));
    HAL_TRY(CudaStatus(cudaMemcpyAsync(h->target.p, target, m * sizeof(float), cudaMemcpyHostToDevice, s),
                       "cudaMemcpy(target)"));
    HAL_TRY(CudaStatus(cudaStreamSynchronize(s), "hal_cuda_adjoint_set_problem"));
    h->hasProblem = true;
    return HAL_CUDA_OK;
}

extern "C" int hal_cuda_adjoint_forward(hal_cuda_adjoint *h, const float *D, double decay, const float *src,
                                        double *loss, float *fT)
{
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr && D != nullptr && loss != nullptr, "hal_cuda_adjoint_forward: NULL argument");
    HAL_REQUIRE(h->hasProblem, "hal_cuda_adjoint_forward: call hal_cuda_adjoint_set_problem first");
    HAL_REQUIRE(std::isfinite(decay), "hal_cuda_adjoint_forward: decay %g", decay);
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    return h->RunForward(D, decay, src, loss, fT);
}

extern "C" int hal_cuda_adjoint_gradient(hal_cuda_adjoint *h, const float *D, double decay, const float *src,
                                         double *loss, float *gradD, double *gradDecay, float *gradSrc)
{
    HAL_TRACE();
    HAL_REQUIRE(h != nullptr && D != nullptr && loss != nullptr, "hal_cuda_adjoint_gradient: NULL argument");
    HAL_REQUIRE(h->hasProblem, "hal_cuda_adjoint_gradient: call hal_cuda_adjoint_set_problem first");
    HAL_REQUIRE(std::isfinite(decay), "hal_cuda_adjoint_gradient: decay %g", decay);
    HAL_TRY(halcuda::CudaStatus(cudaSetDevice(h->device), "cudaSetDevice"));
    return h->RunGradient(D, decay, src, loss, gradD, gradDecay, gradSrc);
}

extern "C" int hal_cuda_adjoint_times(hal_cuda_adjoint *h, float *msForward, float *msGradient)
{
    HAL_REQUIRE(h != nullptr && msForward != nullptr && msGradient != nullptr, "hal_cuda_adjoint_times: NULL argument");
    *msForward = h->msForward;
    *msGradient = h->msGradient;
    return HAL_CUDA_OK;
}
