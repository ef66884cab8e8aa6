// adi_plan.cpp -- FP64 precomputation of the ADI line solves (adi_plan.h).
#include "adi_plan.h"

#include <algorithm>
#include <cmath>

namespace halcuda
{
    namespace
    {
        // Diagonal of row i of a line of length L, as ADISolveRow
        // (ADIequations.h:235-269) and TdmaSolver::TDMAperiodic's adjusted
        // diagonal (TdmaSolver.h:80-95) build it.
        double Diagonal(int32_t i, int32_t L, double offDiag, int ends)
        {
            if (ends == kEndsPeriodic)
            {
                double b = 1 - 2 * offDiag;
                const double gamma = -b;
                if (i == 0)
                {
                    return b - gamma;
                }
                if (i == L - 1)
                {
                    return b - (offDiag * offDiag) / gamma;
                }
                return b;
            }
            double endAdjust = (ends == kEndsDirichlet) ? 1.0 : -1.0;
            double weight = 2.0;
            if (i == 0)
            {
                weight += endAdjust;
            }
            if (i == L - 1)
            {
                weight += endAdjust;
            }
            return 1 - weight * offDiag;
        }

        // Thomas solve of a tridiagonal system with diagonal bd, constant
        // off-diagonals a (below) and c (above).
        void Thomas(const std::vector<double> &bd, double a, double c, std::vector<double> &x)
        {
            size_t n = bd.size();
            std::vector<double> bp(n), dp(n);
            bp[0] = bd[0];
            dp[0] = x[0];
            for (size_t i = 1; i < n; i++)
            {
                double w = a / bp[i - 1];
                bp[i] = bd[i] - w * c;
                dp[i] = x[i] - w * dp[i - 1];
            }
            x[n - 1] = dp[n - 1] / bp[n - 1];
            for (size_t i = n - 1; i-- > 0;)
            {
                x[i] = (dp[i] - c * x[i + 1]) / bp[i];
            }
        }

        // Coefficients of one block whose diagonal is bd (nb = bd.size() rows).
        void BlockCoefficients(const std::vector<double> &bd, double a, double c, float *dst,
                               std::vector<double> &p, std::vector<double> &q,
                               std::vector<double> &fw, std::vector<double> &ib)
        {
            const int32_t nb = static_cast<int32_t>(bd.size());
            std::vector<double> bp(nb);
            fw.assign(nb, 0.0);
            ib.assign(nb, 0.0);
            for (int32_t i = 0; i < kAdiM; i++)
            {
                dst[kCoefFw * kAdiM + i] = 0.0f;
                dst[kCoefIb * kAdiM + i] = 1.0f;
                dst[kCoefCb * kAdiM + i] = 0.0f;
                dst[kCoefP * kAdiM + i] = 0.0f;
                dst[kCoefQ * kAdiM + i] = 0.0f;
            }
            bp[0] = bd[0];
            for (int32_t i = 1; i < nb; i++)
            {
                double w = a / bp[i - 1];
                bp[i] = bd[i] - w * c;
                fw[i] = w;
                dst[kCoefFw * kAdiM + i] = static_cast<float>(w);
            }
            for (int32_t i = 0; i < nb; i++)
            {
                ib[i] = 1.0 / bp[i];
                dst[kCoefIb * kAdiM + i] = static_cast<float>(1.0 / bp[i]);
                if (i < nb - 1)
                {
                    dst[kCoefCb * kAdiM + i] = static_cast<float>(c / bp[i]);
                }
            }
            p.assign(nb, 0.0);
            q.assign(nb, 0.0);
            p[0] = a;
            q[nb - 1] = c;
            Thomas(bd, a, c, p);
            Thomas(bd, a, c, q);
            for (int32_t i = 0; i < nb; i++)
            {
                dst[kCoefP * kAdiM + i] = static_cast<float>(p[i]);
                dst[kCoefQ * kAdiM + i] = static_cast<float>(q[i]);
            }
        }

        // Inverse of a small tridiagonal matrix (column by column).
        void InvertTridiagonal(const std::vector<double> &sub, const std::vector<double> &dia,
                               const std::vector<double> &sup, std::vector<double> &inv)
        {
            size_t n = dia.size();
            inv.assign(n * n, 0.0);
            std::vector<double> bp(n), col(n);
            for (size_t j = 0; j < n; j++)
            {
                for (size_t i = 0; i < n; i++)
                {
                    col[i] = (i == j) ? 1.0 : 0.0;
                }
                bp[0] = dia[0];
                for (size_t i = 1; i < n; i++)
                {
                    double w = sub[i] / bp[i - 1];
                    bp[i] = dia[i] - w * sup[i - 1];
                    col[i] -= w * col[i - 1];
                }
                col[n - 1] /= bp[n - 1];
                for (size_t i = n - 1; i-- > 0;)
                {
                    col[i] = (col[i] - sup[i] * col[i + 1]) / bp[i];
                }
                for (size_t i = 0; i < n; i++)
                {
                    inv[i * n + j] = col[i];
                }
            }
        }
    }

    bool BuildAdiLinePlan(int32_t L, double r, int ends, AdiLinePlanHost &out)
    {
        if (L < 1 || L > kAdiM * kAdiMaxChunks)
        {
            return false;
        }
        out = AdiLinePlanHost();
        out.L = L;
        out.ends = ends;
        const int32_t P = (L + kAdiM - 1) / kAdiM;
        out.P = P;
        const double a = -r / 2.0;
        const double c = a;
        out.offDiag = a;

        std::vector<double> diag(L);
        for (int32_t i = 0; i < L; i++)
        {
            diag[i] = Diagonal(i, L, a, ends);
        }
        // L == 1 periodic: the reference adjusts only the i == 0 branch.

        out.coef.assign(3 * kCoefCount * kAdiM, 0.0f);
        std::vector<double> p[3], q[3], fw[3], ib[3];
        std::vector<int32_t> nbOf(3, 0);
        for (int t = 0; t < 3; t++)
        {
            int32_t first, nb;
            if (P == 1)
            {
                if (t != 0)
                {
                    continue;
                }
                first = 0;
                nb = L;
            }
            else if (t == 0)
            {
                first = 0;
                nb = kAdiM - 1;
            }
            else if (t == 1)
            {
                if (P < 3)
                {
                    continue;
                }
                first = kAdiM;
                nb = kAdiM - 1;
            }
            else
            {
                first = (P - 1) * kAdiM;
                nb = L - first;
            }
            std::vector<double> bd(diag.begin() + first, diag.begin() + first + nb);
            BlockCoefficients(bd, a, c, &out.coef[t * kCoefCount * kAdiM], p[t], q[t], fw[t], ib[t]);
            nbOf[t] = nb;
        }

        // Reduced system over the P-1 separators.
        const int32_t S = P - 1;
        if (S > 0)
        {
            auto typeOf = [&](int32_t k) { return AdiBlockType(k, P); };
            std::vector<double> sub(S, 0.0), dia(S, 0.0), sup(S, 0.0);
            for (int32_t k = 0; k < S; k++)
            {
                int tl = typeOf(k), tr = typeOf(k + 1);
                double bsep = diag[(k + 1) * kAdiM - 1];
                dia[k] = bsep - a * q[tl][nbOf[tl] - 1] - c * p[tr][0];
                if (k >= 1)
                {
                    sub[k] = -a * p[tl][nbOf[tl] - 1];
                }
                if (k <= S - 2)
                {
                    sup[k] = -c * q[tr][0];
                }
            }
            std::vector<double> G;
            InvertTridiagonal(sub, dia, sup, G);
            double gmax = 0.0;
            for (int32_t k = 0; k < S; k++)
            {
                gmax = std::max(gmax, std::fabs(G[k * S + k]));
            }
            const double tol = gmax * std::ldexp(1.0, -46);
            int32_t B = 0;
            for (int32_t k = 0; k < S; k++)
            {
                for (int32_t j = 0; j < S; j++)
                {
                    if (std::fabs(G[k * S + j]) > tol)
                    {
                        B = std::max(B, std::abs(j - k));
                    }
                }
            }
            out.B = B;
            out.gband.assign(static_cast<size_t>(S) * (2 * B + 1), 0.0f);
            for (int32_t k = 0; k < S; k++)
            {
                for (int32_t t = 0; t <= 2 * B; t++)
                {
                    int32_t j = k - B + t;
                    if (j >= 0 && j < S)
                    {
                        out.gband[static_cast<size_t>(k) * (2 * B + 1) + t] = static_cast<float>(G[k * S + j]);
                    }
                }
            }
        }

        // Self-check: run the chunked decomposition (in FP64, with the full
        // reduced inverse) on a test right-hand side and compare with a
        // direct Thomas solve of the whole line.
        {
            std::vector<double> d(L), direct(L), x(L, 0.0);
            for (int32_t i = 0; i < L; i++)
            {
                d[i] = 1.0 + 0.5 * std::sin(0.37 * i) + 0.01 * i;
            }
            direct = d;
            Thomas(diag, a, c, direct);
            std::vector<std::vector<double>> z(P);
            for (int32_t k = 0; k < P; k++)
            {
                int t = AdiBlockType(k, P);
                int32_t nb = nbOf[t];
                z[k].assign(d.begin() + k * kAdiM, d.begin() + k * kAdiM + nb);
                for (int32_t i = 1; i < nb; i++)
                {
                    z[k][i] -= fw[t][i] * z[k][i - 1];
                }
                z[k][nb - 1] *= ib[t][nb - 1];
                for (int32_t i = nb - 1; i-- > 0;)
                {
                    z[k][i] = z[k][i] * ib[t][i] - (c * ib[t][i]) * z[k][i + 1];
                }
            }
            std::vector<double> sep(std::max(S, 1), 0.0), rhs(std::max(S, 1), 0.0);
            for (int32_t k = 0; k < S; k++)
            {
                int tl = AdiBlockType(k, P);
                rhs[k] = d[(k + 1) * kAdiM - 1] - a * z[k][nbOf[tl] - 1] - c * z[k + 1][0];
            }
            for (int32_t k = 0; k < S; k++)
            {
                double acc = 0.0;
                for (int32_t t = 0; t <= 2 * out.B; t++)
                {
                    int32_t j = k - out.B + t;
                    if (j >= 0 && j < S)
                    {
                        acc += static_cast<double>(out.gband[static_cast<size_t>(k) * (2 * out.B + 1) + t]) * rhs[j];
                    }
                }
                sep[k] = acc;
            }
            double err = 0.0, scale = 0.0;
            for (int32_t k = 0; k < P; k++)
            {
                int t = AdiBlockType(k, P);
                double sL = (k >= 1) ? sep[k - 1] : 0.0;
                double sR = (k < S) ? sep[k] : 0.0;
                for (int32_t i = 0; i < nbOf[t]; i++)
                {
                    x[k * kAdiM + i] = z[k][i] - sL * p[t][i] - sR * q[t][i];
                }
                if (k < S)
                {
                    x[(k + 1) * kAdiM - 1] = sR;
                }
            }
            for (int32_t i = 0; i < L; i++)
            {
                err = std::max(err, std::fabs(x[i] - direct[i]));
                scale = std::max(scale, std::fabs(direct[i]));
            }
            out.selfCheck = err / std::max(scale, 1e-300);
        }

        if (ends == kEndsPeriodic)
        {
            // TdmaSolver.h:80-119: gamma = -b, alpha = a (sub-diagonal of row
            // 0), beta = c (super-diagonal of row L-1).
            const double b = 1 - 2 * a;
            const double gamma = -b;
            const double alpha = a;
            const double beta = c;
            std::vector<double> u(L, 0.0);
            for (int32_t i = 0; i < L; i++)
            {
                if (i == 0)
                {
                    u[i] = gamma;
                }
                else if (i == L - 1)
                {
                    u[i] = alpha;
                }
            }
            Thomas(diag, a, c, u);
            out.zsm.resize(L);
            for (int32_t i = 0; i < L; i++)
            {
                out.zsm[i] = static_cast<float>(u[i]);
            }
            out.betaOverGamma = beta / gamma;
            double vz = u[0] + u[L - 1] * out.betaOverGamma;
            out.invDenom = 1.0 / (1.0 + vz);
        }
        return true;
    }
}
