// value.cu — the aerosol value kernel (rt_solver.c:188-235): the
// intensity-to-intensity aerosol phase table of every Fourier mode by direct
// azimuth integration of the tabulated P11,
//     V_m(mu_j, mu_k) = (1/720) sum_q P11(Theta_q) cos(m phi_q),
//     phi_q = 2 pi (q + 1/2) / 720,  cos Theta = mu_j mu_k + s_j s_k cos phi,
// P11 linear in the scattering angle in degrees, clamped to the end values.
// Rows: the sun (mu_j = -mu0, rt_atm.c:244) and the Gauss nodes (+mu_i);
// columns: every ring slot at +mu_o and -mu_o.  The midpoints are symmetric
// about pi, so the 360 pairs (phi, 2 pi - phi) are summed once and doubled.
//
// Precision: the scattering angle comes from the half-angle forms
//     sin^2(Theta/2) = sin^2((t_j - t_k)/2) + s_j s_k sin^2(phi/2)
//     cos^2(Theta/2) = cos^2((t_j + t_k)/2) + s_j s_k cos^2(phi/2)
// (t = acos(mu) in FP64 once per pair), which have no cancellation at the
// forward or backward peak, so FP32 carries Theta to ~1e-7 relative; the
// products accumulate in FP32 over blocks of 45 azimuths and the blocks in
// FP64; cos(m phi) comes from a shared table made with cospif of the exact
// reduced argument.
//
// One block of 128 threads per (pixel, 128 (row, column) pairs); the block
// holds the pixel's table, a 4096-bucket angle index for O(1) bracketing,
// the azimuth factors and the cosine table of one chunk of 32 modes.
#include "kernels.cuh"

#define VK_NQ 360           // azimuth pairs of the 720-point midpoint rule
#define VK_MC 32            // modes per chunk
#define VK_NB 4096          // angle buckets over 0 .. 180 degrees

size_t value_kernel_smem_bytes(int n_ang)
{
    return sizeof(float) * (2 * (size_t)n_ang + 2 * VK_NQ + (size_t)VK_NQ * VK_MC) + sizeof(int) * VK_NB;
}

__global__ void __launch_bounds__(128) k_value_pfm(const PixDev *px, int p0, Geom G, const double *gmu,
                                                   const double *vk_th, const double *vk_p11, float *V,
                                                   long long vstride)
{
    const int pp = blockIdx.y, p = p0 + pp;
    const PixDev &d = px[p];
    const int n = d.vk_n;
    if (n < 2) return;
    extern __shared__ float vk_smem[];
    float *th = vk_smem, *pt = th + n;                  // table (ascending degrees, P11)
    float *sh2 = pt + n, *ch2 = sh2 + VK_NQ;            // sin^2(phi/2), cos^2(phi/2)
    float *ct = ch2 + VK_NQ;                            // [VK_NQ][VK_MC] cos(m phi) of the chunk
    int *bk = (int *)(ct + VK_NQ * VK_MC);              // [VK_NB] last node at or below the bucket start
    const int tid = threadIdx.x;
    for (int i = tid; i < n; i += blockDim.x) {
        th[i] = (float)vk_th[d.vk_off + i];
        pt[i] = (float)vk_p11[d.vk_off + i];
    }
    for (int q = tid; q < VK_NQ; q += blockDim.x) {
        // phi = 2 pi (q + 1/2) / 720: phi / 2 = pi (2q + 1) / 1440
        float sp, cp;
        sincospif((2.0f * q + 1.0f) / 1440.0f, &sp, &cp);
        sh2[q] = sp * sp;
        ch2[q] = cp * cp;
    }
    __syncthreads();
    for (int b = tid; b < VK_NB; b += blockDim.x) {
        const float x = 180.0f * (float)b / (float)VK_NB;
        int lo = 0, hi = n - 1;
        if (x < th[0]) { bk[b] = 0; continue; }
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (th[mid] <= x) lo = mid; else hi = mid;
        }
        bk[b] = lo;
    }
    // this thread's (row, column) pair
    const int N = G.N, NR = G.NR, npair = (N + 1) * 2 * NR;
    const int e = blockIdx.x * blockDim.x + tid;
    const bool mine = e < npair;
    const int a = mine ? e / (2 * NR) : 0, bcol = mine ? e - a * 2 * NR : 0;
    const int o = bcol < NR ? bcol : bcol - NR;
    const double mj = a == 0 ? -d.mu0 : gmu[a - 1];
    const double mo = ring_mu(d, gmu, N, o), mk = bcol < NR ? mo : -mo;
    const double tj = acos(fmin(1.0, fmax(-1.0, mj))), tk = acos(fmin(1.0, fmax(-1.0, mk)));
    const double sd = sin(0.5 * (tj - tk)), cs = cos(0.5 * (tj + tk));
    const float A = (float)(sd * sd), Bc = (float)(cs * cs);
    const float K = (float)(sqrt(fmax(0.0, 1.0 - mj * mj)) * sqrt(fmax(0.0, 1.0 - mk * mk)));
    const float rad2deg = (float)(360.0 / OCRT_PI);   // 2 x (180 / pi): Theta = 2 atan2(...)
    const float nbk = (float)VK_NB / 180.0f;
    float *Vp = V + (size_t)pp * vstride;
    const int M = d.M;
    for (int m0 = 0; m0 <= M; m0 += VK_MC) {
        const int mc = min(VK_MC, M + 1 - m0);
        __syncthreads();
        for (int x = tid; x < VK_NQ * VK_MC; x += blockDim.x) {
            const int q = x / VK_MC, j = x - q * VK_MC;
            // cos(m phi_q) = cospi(m (2q + 1) / 720), the argument reduced mod 2 exactly
            const int r = ((m0 + j) * (2 * q + 1)) % 1440;
            ct[x] = cospif((float)r / 720.0f);
        }
        __syncthreads();
        if (!mine) continue;
        double acc[VK_MC];
#pragma unroll
        for (int j = 0; j < VK_MC; ++j) acc[j] = 0.0;
        for (int q0 = 0; q0 < VK_NQ; q0 += 45) {
            float part[VK_MC];
#pragma unroll
            for (int j = 0; j < VK_MC; ++j) part[j] = 0.f;
            for (int q = q0; q < q0 + 45; ++q) {
                const float s2 = A + K * sh2[q], c2 = Bc + K * ch2[q];
                const float tdeg = rad2deg * atan2f(sqrtf(s2), sqrtf(c2));
                float P;
                if (tdeg <= th[0]) {
                    P = pt[0];
                } else if (tdeg >= th[n - 1]) {
                    P = pt[n - 1];
                } else {
                    int lo = bk[min(VK_NB - 1, (int)(tdeg * nbk))];
                    while (lo > 0 && th[lo] > tdeg) --lo;            // bucket start rounded past tdeg
                    while (lo + 1 < n - 1 && th[lo + 1] <= tdeg) ++lo;
                    const float t = (tdeg - th[lo]) / (th[lo + 1] - th[lo]);
                    P = pt[lo] + t * (pt[lo + 1] - pt[lo]);
                }
                const float *cq = ct + q * VK_MC;
#pragma unroll
                for (int j = 0; j < VK_MC; ++j) part[j] = fmaf(P, cq[j], part[j]);
            }
#pragma unroll
            for (int j = 0; j < VK_MC; ++j) acc[j] += (double)part[j];
        }
        for (int j = 0; j < mc; ++j)
            Vp[((size_t)(m0 + j) * (N + 1) + a) * 2 * NR + bcol] = (float)(acc[j] * (2.0 / 720.0));
    }
}
