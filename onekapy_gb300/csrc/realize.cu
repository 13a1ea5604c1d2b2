// realize.cu -- realization draw, weighted least-squares fit and MVN draw (FP64).
//
// One warp per realization.  References (paths within OnekaPy):
//   oneka/stochastic.py:224-241    per-realization draws of Q_i, K, n, H; fit; MVN draw
//   oneka/stochastic.py:274-342    generate_random_variate / compute_variate_mean
//   oneka/model.py:497-567         construct_fit: FOSM potentials and weighted rows
//   oneka/model.py:571-606         compute_fit: lstsq + inv(WA^T WA)
//
// Differences by design (the reference is unseeded and non-reproducible):
//   * variates come from Philox4x32-10 (Salmon et al., SC'11), counter =
//     (variate index, realization index lo/hi, "ONEK"), key = seed, so any
//     realization can be drawn independently of the others and of the shard;
//   * the fit solves the 6x6 normal equations WA^T WA c = WA^T Wb with a
//     Jacobi-scaled Cholesky factor L (the reference's lstsq uses an SVD; both
//     give the least-squares solution); the covariance is its inverse, as in
//     the reference, and the MVN draw is mean + D L^-T z, whose covariance is
//     exactly (WA^T WA)^-1 (numpy's multivariate_normal uses an SVD of it).
#include <math.h>

#include "oneka_internal.cuh"

namespace oneka {
namespace {

constexpr uint32_t kPhiloxM0 = 0xD2511F53u, kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u, kPhiloxW1 = 0xBB67AE85u;
constexpr uint32_t kStreamTag = 0x4F4E454Bu;
constexpr double kPi = 3.141592653589793;

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int i = 0; i < 10; ++i) {
        const uint32_t hi0 = __umulhi(kPhiloxM0, c.x), lo0 = kPhiloxM0 * c.x;
        const uint32_t hi1 = __umulhi(kPhiloxM1, c.z), lo1 = kPhiloxM1 * c.z;
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
        k0 += kPhiloxW0;
        k1 += kPhiloxW1;
    }
    return c;
}

__device__ __forceinline__ double u53(uint32_t hi, uint32_t lo) {
    const unsigned long long v = ((unsigned long long)hi << 32) | lo;
    return (double)(v >> 11) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ void uniforms(unsigned long long seed, unsigned long long real, uint32_t var,
                                         double& u0, double& u1) {
    const uint4 w = philox4x32_10(make_uint4(var, (uint32_t)real, (uint32_t)(real >> 32), kStreamTag),
                                  (uint32_t)seed, (uint32_t)(seed >> 32));
    u0 = u53(w.x, w.y);
    u1 = u53(w.z, w.w);
}

__device__ double variate(const OnekaDist& d, double u0, double u1) {
    switch (d.kind) {
        case ONEKA_DIST_UNIFORM:
            return d.p0 + (d.p1 - d.p0) * u0;
        case ONEKA_DIST_TRIANGULAR: {
            const double a = d.p0, c = d.p1, b = d.p2;
            if (b - a <= 0.0) return a;
            const double fc = (c - a) / (b - a);
            if (u0 < fc) return a + sqrt(u0 * (b - a) * (c - a));
            return b - sqrt((1.0 - u0) * (b - a) * (b - c));
        }
        case ONEKA_DIST_LOGNORMAL: {
            const double z = sqrt(-2.0 * log(1.0 - u0)) * cos(2.0 * kPi * u1);
            return exp(d.p0 + d.p1 * z);
        }
        default:
            return d.p0;
    }
}

// compute_variate_mean (stochastic.py:310-342), plus the lognormal mean.
__device__ double variate_mean(const OnekaDist& d) {
    switch (d.kind) {
        case ONEKA_DIST_UNIFORM: return (d.p0 + d.p1) / 2.0;
        case ONEKA_DIST_TRIANGULAR: return (d.p0 + d.p1 + d.p2) / 3.0;
        case ONEKA_DIST_LOGNORMAL: return exp(d.p0 + 0.5 * d.p1 * d.p1);
        default: return d.p0;
    }
}

// One weighted row of the least-squares problem (model.py:545-565): the
// FOSM potential of observation ob = (x, y, z_ev, z_std) under base, K, H,
// less the wells' potential pw there, both over the potential's standard
// deviation.  Returns false where the reference raises RangeError (a head at
// or below the base).
__device__ __forceinline__ bool fosm_row(const double* ob, double base, double K, double H, double xo,
                                         double yo, double pw, double a[6], double& bo) {
    const double x = ob[0], y = ob[1], z_ev = ob[2], z_std = ob[3];
    const double head = z_ev - base;
    double pot_ev, pot_std;
    if (head >= H) {
        pot_ev = (K * H * (head - 0.5 * H));
        pot_std = K * H * z_std;
    } else if (head > 0) {
        pot_ev = (0.5 * K * (head * head + z_std * z_std));
        pot_std = K * head * z_std;
    } else {
        return false;
    }
    const double dx = x - xo, dy = y - yo;
    a[0] = dx * dx / pot_std;
    a[1] = dy * dy / pot_std;
    a[2] = dx * dy / pot_std;
    a[3] = dx / pot_std;
    a[4] = dy / pot_std;
    a[5] = 1.0 / pot_std;
    bo = (pot_ev - pw) / pot_std;
    return true;
}

// N += a a^T (lower triangle, row by row), b += a bo.
__device__ __forceinline__ void accumulate_normal(const double a[6], double bo, double N[21], double b[6]) {
    int t = 0;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
#pragma unroll
        for (int j = 0; j <= i; ++j) N[t++] += a[i] * a[j];
        b[i] += a[i] * bo;
    }
}

// Sum the lanes' normal equations (butterfly: every lane ends with the total).
__device__ __forceinline__ void warp_reduce_normal(double N[21], double b[6], int& bad) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int i = 0; i < 21; ++i) N[i] += __shfl_xor_sync(0xffffffffu, N[i], off);
#pragma unroll
        for (int i = 0; i < 6; ++i) b[i] += __shfl_xor_sync(0xffffffffu, b[i], off);
        bad |= __shfl_xor_sync(0xffffffffu, bad, off);
    }
}

// The least-squares solution and covariance from the normal equations
// N c = b (model.py:597-604: lstsq(WA, Wb) and inv(WA^T WA)): Jacobi scaling
// D = diag(N)^-1/2, Cholesky factor L of D N D, c = D L^-T L^-1 D b and
// cov = D L^-T L^-1 D.  Returns ONEKA_REAL_OK or ONEKA_REAL_NOT_SPD (then ev
// and cov are NaN).  L and d are kept for the MVN draw.
__device__ int solve_normal(const double N[21], const double b[6], double L[6][6], double d[6], double ev[6],
                            double cov[6][6]) {
    int status = ONEKA_REAL_OK;
    double A[6][6];
    {
        int t = 0;
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j <= i; ++j) { A[i][j] = N[t]; A[j][i] = N[t]; ++t; }
    }
    for (int i = 0; i < 6; ++i) {
        ev[i] = 0.0;
        if (!(A[i][i] > 0.0)) status = ONEKA_REAL_NOT_SPD;
        d[i] = (A[i][i] > 0.0) ? 1.0 / sqrt(A[i][i]) : 0.0;
    }
    if (status == ONEKA_REAL_OK) {
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) A[i][j] *= d[i] * d[j];
        for (int j = 0; j < 6 && status == ONEKA_REAL_OK; ++j) {
            double s = A[j][j];
            for (int k = 0; k < j; ++k) s -= L[j][k] * L[j][k];
            if (!(s > 1e-14)) { status = ONEKA_REAL_NOT_SPD; break; }
            L[j][j] = sqrt(s);
            for (int i = j + 1; i < 6; ++i) {
                double v = A[i][j];
                for (int k = 0; k < j; ++k) v -= L[i][k] * L[j][k];
                L[i][j] = v / L[j][j];
            }
            for (int i = 0; i < j; ++i) L[i][j] = 0.0;
        }
    }
    if (status != ONEKA_REAL_OK) {
        for (int i = 0; i < 6; ++i) {
            ev[i] = NAN;
            for (int j = 0; j < 6; ++j) cov[i][j] = NAN;
        }
        return status;
    }
    double y[6], z[6];
    for (int i = 0; i < 6; ++i) {                 // L y = D b
        double v = b[i] * d[i];
        for (int k = 0; k < i; ++k) v -= L[i][k] * y[k];
        y[i] = v / L[i][i];
    }
    for (int i = 5; i >= 0; --i) {                // L^T z = y
        double v = y[i];
        for (int k = i + 1; k < 6; ++k) v -= L[k][i] * z[k];
        z[i] = v / L[i][i];
    }
    for (int i = 0; i < 6; ++i) ev[i] = d[i] * z[i];
    // covariance (WA^T WA)^-1 = D L^-T L^-1 D
    double Li[6][6];
    for (int j = 0; j < 6; ++j) {
        for (int i = 0; i < 6; ++i) {
            double v = (i == j) ? 1.0 : 0.0;
            for (int k = 0; k < i; ++k) v -= L[i][k] * Li[k][j];
            Li[i][j] = (i < j) ? 0.0 : v / L[i][i];
        }
    }
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            double v = 0.0;
            for (int k = (i > j ? i : j); k < 6; ++k) v += Li[k][i] * Li[k][j];
            cov[i][j] = d[i] * d[j] * v;
        }
    return status;
}

struct RealizeParams {
    OnekaSite site;
    const OnekaDist* qdist;
    OnekaDist adist[3];
    const double* logr2;
    unsigned long long seed, first;
    int nreal, mode;
    OnekaRealizations out;
};

constexpr int kWarps = 4;

__global__ void __launch_bounds__(32 * kWarps) realize_kernel(const RealizeParams P) {
    extern __shared__ double qsm[];                 // [kWarps][nwells]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * kWarps + warp;
    if (r >= P.nreal) return;
    const int nw = P.site.nwells;
    double* q = qsm + warp * nw;
    const unsigned long long rg = P.first + (unsigned long long)r;
    const bool given = (P.mode == ONEKA_MODE_GIVEN || P.mode == ONEKA_MODE_GIVEN_EV);
    const bool draw_coef = (P.mode == ONEKA_MODE_STOCHASTIC || P.mode == ONEKA_MODE_GIVEN);

    // (1) well discharges, then K, porosity, thickness (stochastic.py:224-233)
    for (int w = lane; w < nw; w += 32) {
        double v;
        if (given) {
            v = P.out.q[(long long)r * nw + w];
        } else if (P.mode == ONEKA_MODE_MEAN) {
            v = variate_mean(P.qdist[w]);
        } else {
            double u0, u1;
            uniforms(P.seed, rg, (uint32_t)w, u0, u1);
            v = variate(P.qdist[w], u0, u1);
        }
        q[w] = v;
        if (!given) P.out.q[(long long)r * nw + w] = v;
    }
    double aq[3];
    for (int a = 0; a < 3; ++a) {
        if (given) {
            aq[a] = P.out.aquifer[3LL * r + a];
        } else if (P.mode == ONEKA_MODE_MEAN) {
            aq[a] = variate_mean(P.adist[a]);
        } else {
            double u0, u1;
            uniforms(P.seed, rg, (uint32_t)(nw + a), u0, u1);
            aq[a] = variate(P.adist[a], u0, u1);
        }
    }
    __syncwarp();
    const double K = aq[0], H = aq[2];

    // (2) FOSM rows and normal equations (model.py:545-565), lanes over observations
    double N[21], b[6];
#pragma unroll
    for (int i = 0; i < 21; ++i) N[i] = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) b[i] = 0.0;
    int bad = 0;
    for (int o = lane; o < P.site.nobs; o += 32) {
        const double* ob = P.site.obs + 4LL * o;
        double pw = 0.0;
        for (int w = 0; w < nw; ++w) {
            double l2;
            if (P.logr2) {
                l2 = P.logr2[(long long)o * nw + w];
            } else {
                const double ddx = ob[0] - P.site.wells[3 * w], ddy = ob[1] - P.site.wells[3 * w + 1];
                l2 = log(ddx * ddx + ddy * ddy);
            }
            pw += q[w] * l2 * 0.07957747154594767;
        }
        double a[6], bo;
        if (!fosm_row(ob, P.site.base, K, H, P.site.xo, P.site.yo, pw, a, bo)) {
            bad = 1;
            continue;
        }
        accumulate_normal(a, bo, N, b);
    }
    warp_reduce_normal(N, b, bad);
    if (lane != 0) return;

    double L[6][6], d[6], ev[6], cov[6][6];
    int status = bad ? ONEKA_REAL_RANGE : solve_normal(N, b, L, d, ev, cov);
    double coef[6] = {0, 0, 0, 0, 0, 0};
    if (status == ONEKA_REAL_OK) {
        // (4) multivariate-normal draw (stochastic.py:240-241): mean + D L^-T g
        if (draw_coef) {
            double g[6];
            for (int pr = 0; pr < 3; ++pr) {
                double u0, u1;
                uniforms(P.seed, rg, (uint32_t)(nw + 3 + pr), u0, u1);
                const double rad = sqrt(-2.0 * log(1.0 - u0));
                g[2 * pr] = rad * cos(2.0 * kPi * u1);
                g[2 * pr + 1] = rad * sin(2.0 * kPi * u1);
            }
            double w[6];
            for (int i = 5; i >= 0; --i) {
                double v = g[i];
                for (int k = i + 1; k < 6; ++k) v -= L[k][i] * w[k];
                w[i] = v / L[i][i];
            }
            for (int i = 0; i < 6; ++i) coef[i] = ev[i] + d[i] * w[i];
        } else {
            for (int i = 0; i < 6; ++i) coef[i] = ev[i];
        }
        for (int i = 0; i < 6; ++i)
            if (!isfinite(ev[i]) || !isfinite(coef[i])) status = ONEKA_REAL_NOT_FINITE;
    } else {
        for (int i = 0; i < 6; ++i) {
            coef[i] = ev[i] = NAN;
            for (int j = 0; j < 6; ++j) cov[i][j] = NAN;
        }
    }
    for (int i = 0; i < 6; ++i) P.out.coef[6LL * r + i] = coef[i];
    if (P.out.coef_ev)
        for (int i = 0; i < 6; ++i) P.out.coef_ev[6LL * r + i] = ev[i];
    if (P.out.coef_cov)
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) P.out.coef_cov[36LL * r + 6 * i + j] = cov[i][j];
    if (!given)
        for (int a = 0; a < 3; ++a) P.out.aquifer[3LL * r + a] = aq[a];
    if (P.out.status) P.out.status[r] = status;
}

// construct_fit for one model (model.py:545-565): one thread per observation.
__global__ void fit_rows_kernel(const OnekaSite site, const double* __restrict__ q, double K, double H,
                                double* __restrict__ WA, double* __restrict__ Wb, int32_t* __restrict__ status) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= site.nobs) return;
    const double* ob = site.obs + 4LL * o;
    double pw = 0.0;                                   // compute_potential_wells_only (model.py:258-264)
    for (int w = 0; w < site.nwells; ++w) {
        const double ddx = ob[0] - site.wells[3 * w], ddy = ob[1] - site.wells[3 * w + 1];
        pw += q[w] * log(ddx * ddx + ddy * ddy) * 0.07957747154594767;
    }
    double a[6], bo;
    if (!fosm_row(ob, site.base, K, H, site.xo, site.yo, pw, a, bo)) {
        for (int i = 0; i < 6; ++i) WA[6LL * o + i] = NAN;
        Wb[o] = NAN;
        atomicMax(status, ONEKA_REAL_RANGE);
        return;
    }
    for (int i = 0; i < 6; ++i) WA[6LL * o + i] = a[i];
    Wb[o] = bo;
}

// compute_fit (model.py:597-604) for nfit independent problems of nobs rows:
// one warp per problem, lanes over the rows.
__global__ void fit_solve_kernel(const double* __restrict__ WA, const double* __restrict__ Wb, int nobs,
                                 int nfit, double* __restrict__ coef_ev, double* __restrict__ coef_cov,
                                 int32_t* __restrict__ status) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int f = blockIdx.x * kWarps + warp;
    if (f >= nfit) return;
    double N[21], b[6];
#pragma unroll
    for (int i = 0; i < 21; ++i) N[i] = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) b[i] = 0.0;
    int bad = 0;
    for (int o = lane; o < nobs; o += 32) {
        const double* row = WA + (6LL * nobs) * f + 6LL * o;
        double a[6];
        for (int i = 0; i < 6; ++i) a[i] = row[i];
        const double bo = Wb[(long long)nobs * f + o];
        bool fin = isfinite(bo);
        for (int i = 0; i < 6; ++i) fin = fin && isfinite(a[i]);
        if (!fin) {
            bad = 1;
            continue;
        }
        accumulate_normal(a, bo, N, b);
    }
    warp_reduce_normal(N, b, bad);
    if (lane != 0) return;
    double L[6][6], d[6], ev[6], cov[6][6];
    int st = bad ? ONEKA_REAL_NOT_FINITE : solve_normal(N, b, L, d, ev, cov);
    if (bad)
        for (int i = 0; i < 6; ++i) {
            ev[i] = NAN;
            for (int j = 0; j < 6; ++j) cov[i][j] = NAN;
        }
    for (int i = 0; i < 6; ++i) coef_ev[6LL * f + i] = ev[i];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) coef_cov[36LL * f + 6 * i + j] = cov[i][j];
    if (status) status[f] = st;
}

__global__ void logr2_kernel(OnekaSite site, double* __restrict__ logr2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)site.nobs * site.nwells) return;
    const int o = (int)(i / site.nwells), w = (int)(i % site.nwells);
    const double dx = site.obs[4LL * o] - site.wells[3 * w];
    const double dy = site.obs[4LL * o + 1] - site.wells[3 * w + 1];
    logr2[i] = log(dx * dx + dy * dy);
}

}  // namespace

cudaError_t launch_realize(const OnekaSite& site, const OnekaDist* qdist, const OnekaDist* adist,
                           const double* logr2, unsigned long long seed, unsigned long long first,
                           int nreal, int mode, const OnekaRealizations& out, cudaStream_t s) {
    if (nreal <= 0) return cudaSuccess;
    RealizeParams P;
    P.site = site;
    P.qdist = qdist;
    for (int a = 0; a < 3; ++a) P.adist[a] = adist[a];
    P.logr2 = logr2;
    P.seed = seed;
    P.first = first;
    P.nreal = nreal;
    P.mode = mode;
    P.out = out;
    const unsigned blocks = (unsigned)((nreal + kWarps - 1) / kWarps);
    const size_t smem = sizeof(double) * kWarps * (size_t)(site.nwells > 0 ? site.nwells : 1);
    realize_kernel<<<blocks, 32 * kWarps, smem, s>>>(P);
    return cudaGetLastError();
}

cudaError_t launch_fit_rows(const OnekaSite& site, const double* q, double K, double H, double* WA, double* Wb,
                            int32_t* status, cudaStream_t s) {
    if (site.nobs <= 0) return cudaSuccess;
    fit_rows_kernel<<<(unsigned)((site.nobs + 127) / 128), 128, 0, s>>>(site, q, K, H, WA, Wb, status);
    return cudaGetLastError();
}

cudaError_t launch_fit_solve(const double* WA, const double* Wb, int nobs, int nfit, double* coef_ev,
                             double* coef_cov, int32_t* status, cudaStream_t s) {
    if (nfit <= 0) return cudaSuccess;
    fit_solve_kernel<<<(unsigned)((nfit + kWarps - 1) / kWarps), 32 * kWarps, 0, s>>>(WA, Wb, nobs, nfit, coef_ev,
                                                                                      coef_cov, status);
    return cudaGetLastError();
}

cudaError_t launch_logr2(const OnekaSite& site, double* logr2, cudaStream_t s) {
    const long long n = (long long)site.nobs * site.nwells;
    if (n <= 0) return cudaSuccess;
    logr2_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(site, logr2);
    return cudaGetLastError();
}

}  // namespace oneka
