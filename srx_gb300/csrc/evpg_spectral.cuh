// Spectral chain of one equilibrium iteration: forward 3-D FFT of the six
// stress components, Green-operator contraction, inverse 3-D FFT of the nine
// displacement-gradient corrections and the update
//   DisGrad += dDisGradAvg + Re(IFFT(Gamma:FFT(sig)))/N
// (evolution.c:1157-1201; Gamma from CalcGAMMA, init.c:542-592).
//
// Five kernels, each one HBM round trip over its data:
//   fwd_z   real sig pairs -> one complex FFT per pair along z -> half spectra
//   fwd_y   c2c along y
//   x_green c2c along x, Gamma contraction (6 -> 9 components), inverse along x
//   inv_y   c2c along y
//   inv_z   pairs of Hermitian half spectra -> one complex IFFT -> two real
//           fields, fused with the DisGrad update
// The reference keeps Re() of a full complex IFFT of a spectrum that is not
// Hermitian on the Nyquist planes (there n(-k) != -n(k)); x_green feeds the
// half-spectrum transforms the Hermitian part (X(k) + conj X(-k))/2, whose
// inverse is exactly that real part.
#pragma once
#include "evpg_common.cuh"
#include "evpg_fft.cuh"

namespace evpg {

// k-space unit vector, init.c:780-797 (TWO_PI as the reference writes it).
// rn: (T)(1.0/n_a) of the three axes, rounded once on the host; used by the
// FP32 kernels (no FP64 division there), the FP64 kernels divide as written.
template <typename T>
__device__ __forceinline__ void kvec(int kx, int ky, int kz, const Grid& g, const T rn[3], T n[3]) {
    T t[3];
    if (sizeof(T) == 8) {
        t[0] = (T)kx * (T)(1.0 / g.n0);
        t[1] = (T)ky * (T)(1.0 / g.n1);
        t[2] = (T)kz * (T)(1.0 / g.n2);
    } else {
        t[0] = (T)kx * rn[0];
        t[1] = (T)ky * rn[1];
        t[2] = (T)kz * rn[2];
    }
#pragma unroll
    for (int m = 0; m < 3; m++) {
        t[m] -= round(t[m]);
        t[m] *= (T)6.28318530718;
    }
    const T g2 = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    const T s = (T)1 / g2;
#pragma unroll
    for (int m = 0; m < 3; m++) n[m] = t[m] * s;
}

// du = Gamma(k) : sig_hat, returned as 6 B-basis components of its symmetric
// part and A12, A13, A23 of its antisymmetric part. Gamma_ijkl = -Omega_ik n_j n_l
// with Omega = (C0_ijkl n_j n_l)^-1, so du_ij = -n_j (Omega (sig n))_i.
// C0 element access: from the kernel's constant bank (single-RVE kernels) or
// from shared memory re-read at every use (batched kernels; a cached copy
// would pin 81 values in registers).
template <typename T> struct C0Param {
    const T (&c)[3][3][3][3];
    __device__ __forceinline__ T operator()(int i, int j, int k, int l) const { return c[i][j][k][l]; }
};
template <typename T> struct C0Shared {
    const volatile T* c;
    __device__ __forceinline__ T operator()(int i, int j, int k, int l) const { return c[((i * 3 + j) * 3 + k) * 3 + l]; }
};

template <typename T, typename C0>
__device__ __forceinline__ void green_du(const C0& c0, const T n[3], const C2<T> sb[6],
                                         C2<T> out[9]) {
    T sr[3][3], si[3][3];
    {
        T vr[6], vi[6];
#pragma unroll
        for (int c = 0; c < 6; c++) { vr[c] = sb[c].x; vi[c] = sb[c].y; }
        b6_to_sym<T>(vr, sr);
        b6_to_sym<T>(vi, si);
    }
    T nn[3][3], a[3][3];
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
        for (int l = 0; l < 3; l++) nn[j][l] = n[j] * n[l];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = i; k < 3; k++) {
            T s = 0;
#pragma unroll
            for (int j = 0; j < 3; j++)
#pragma unroll
                for (int l = 0; l < 3; l++) s += c0(i, j, k, l) * nn[j][l];
            a[i][k] = s;
            a[k][i] = s;
        }
    T om[3][3];
    om[0][0] = a[1][1] * a[2][2] - a[1][2] * a[2][1];
    om[0][1] = a[0][2] * a[2][1] - a[0][1] * a[2][2];
    om[0][2] = a[0][1] * a[1][2] - a[0][2] * a[1][1];
    om[1][0] = a[1][2] * a[2][0] - a[1][0] * a[2][2];
    om[1][1] = a[0][0] * a[2][2] - a[0][2] * a[2][0];
    om[1][2] = a[0][2] * a[1][0] - a[0][0] * a[1][2];
    om[2][0] = a[1][0] * a[2][1] - a[1][1] * a[2][0];
    om[2][1] = a[0][1] * a[2][0] - a[0][0] * a[2][1];
    om[2][2] = a[0][0] * a[1][1] - a[0][1] * a[1][0];
    const T det = a[0][0] * om[0][0] + a[0][1] * om[1][0] + a[0][2] * om[2][0];
    const T idet = (T)1 / det;
    T tr[3], ti[3], ur[3], ui[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        tr[k] = sr[k][0] * n[0] + sr[k][1] * n[1] + sr[k][2] * n[2];
        ti[k] = si[k][0] * n[0] + si[k][1] * n[1] + si[k][2] * n[2];
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
        ur[i] = (om[i][0] * tr[0] + om[i][1] * tr[1] + om[i][2] * tr[2]) * idet;
        ui[i] = (om[i][0] * ti[0] + om[i][1] * ti[1] + om[i][2] * ti[2]) * idet;
    }
    const T r2 = (T)RSQ2, r3 = (T)RSQ3, r6 = (T)RSQ6, h = (T)0.5;
    T o_r[9], o_i[9];
    // du_ij = -u_i n_j, once for the real and once for the imaginary part
#pragma unroll
    for (int part = 0; part < 2; part++) {
        const T* u = part ? ui : ur;
        T* o = part ? o_i : o_r;
        const T d00 = -u[0] * n[0], d11 = -u[1] * n[1], d22 = -u[2] * n[2];
        const T d01 = -u[0] * n[1], d10 = -u[1] * n[0], d02 = -u[0] * n[2];
        const T d20 = -u[2] * n[0], d12 = -u[1] * n[2], d21 = -u[2] * n[1];
        o[0] = r2 * (d11 - d00);
        o[1] = r6 * ((T)2 * d22 - d00 - d11);
        o[2] = r2 * (d12 + d21);
        o[3] = r2 * (d02 + d20);
        o[4] = r2 * (d01 + d10);
        o[5] = r3 * (d00 + d11 + d22);
        o[6] = h * (d01 - d10);
        o[7] = h * (d02 - d20);
        o[8] = h * (d12 - d21);
    }
#pragma unroll
    for (int c = 0; c < 9; c++) out[c] = mk<T>(o_r[c], o_i[c]);
}

// k = 0 (init.c:558-569): Gamma = -S0 for ElastBC 0, else 0.
template <typename T>
__device__ __forceinline__ void green_k0(const T s0[3][3][3][3], int elast_bc, const C2<T> sb[6],
                                         C2<T> out[9]) {
    if (elast_bc != 0) {
#pragma unroll
        for (int c = 0; c < 9; c++) out[c] = mk<T>((T)0, (T)0);
        return;
    }
    T vr[6], vi[6], sr[3][3], si[3][3], dr[3][3], di[3][3];
#pragma unroll
    for (int c = 0; c < 6; c++) { vr[c] = sb[c].x; vi[c] = sb[c].y; }
    b6_to_sym<T>(vr, sr);
    b6_to_sym<T>(vi, si);
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            T a = 0, b = 0;
#pragma unroll
            for (int k = 0; k < 3; k++)
#pragma unroll
                for (int l = 0; l < 3; l++) {
                    a -= s0[i][j][k][l] * sr[k][l];
                    b -= s0[i][j][k][l] * si[k][l];
                }
            dr[i][j] = a;
            di[i][j] = b;
        }
    T o_r[6], o_i[6];
    sym_to_b6<T>(dr, o_r);
    sym_to_b6<T>(di, o_i);
#pragma unroll
    for (int c = 0; c < 6; c++) out[c] = mk<T>(o_r[c], o_i[c]);
    out[6] = mk<T>((T)0.5 * (dr[0][1] - dr[1][0]), (T)0.5 * (di[0][1] - di[1][0]));
    out[7] = mk<T>((T)0.5 * (dr[0][2] - dr[2][0]), (T)0.5 * (di[0][2] - di[2][0]));
    out[8] = mk<T>((T)0.5 * (dr[1][2] - dr[2][1]), (T)0.5 * (di[1][2] - di[2][1]));
}

}  // namespace evpg
