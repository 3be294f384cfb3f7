// adjoint.cuh -- discrete adjoint of the fluid step on a prescribed rigid mask (FP64).
//
// Forward map of one step (NavierStokes.f90:422-508 with cal_nlk :9-177 and the velocity of
// pressure :273-290), in the half-spectrum representation of the device (S(kx, ky), kx in
// [0, nx/2), ky all, the ky = ny/2 row zero):
//   u = Phi(i ky Pi W) + U,  v = -Phi(i kx Pi W) + V,  wx = Phi(i kx W),  wy = Phi(i ky W)
//   N = F(-(u wx + v wy)) + i kx F(-chi v) - i ky F(-chi u)
//   W' = (W + b10 N + b11 M) E D,  M' = N E           (Euler start-up: W' = (W + dt N) E D)
//   drag' = dx dy sum_window chi u',  lift' = dx dy sum_window chi v'
// with F the forward transform (1/(nx ny), Nyquist row dropped), Phi the inverse (Im of the
// kx = 0 column ignored, X[nx/2] = 0), Pi = 1/|k|^2 (0 at k = 0), E = exp(-nu dt |k|^2), D the
// 2/3 rule.  Their exact transposes, in the real-pair inner product over the stored modes:
//   Phi^T g = nx ny (1 + [kx > 0]) F_unfiltered(g)        (F zeroes the Nyquist row: so does Phi)
//   F^T l   = Phi(w l) / (nx ny),  w = 1 at kx = 0, 1/2 else
//   (multiplication by m)^T = multiplication by conj(m)
// The kernels below are the pointwise parts; the transforms are the ordinary transform kernels.
#pragma once

#include "fluid.cuh"

namespace fsibe {

struct AdjArgs {
    Geometry g;
    const double* etab;  // exp(coefx kx^2) [hx], exp(coefy ky^2) [ny/2+1]
    const int* dcut;
    double b10, b11, dt, c_obj;
    int euler;
    C2<double> *lW, *lM, *lN, *q, *X0, *X1, *X2, *G1, *G2, *G3, *G4, *Gd, *Wn, *Mn;
    const double *u, *v, *wx, *wy, *lnl, *lp1, *lp2, *mask;
    double *lu, *lv, *lwx, *lwy, *gmask, *ubar, *part;
    const DevScalars* S;
    double* J;
    int comp;            // the objective's force component: 0 drag (Force(1)), 1 lift (Force(2))
};

__device__ __forceinline__ void adj_mode(const Geometry& g, int i, int& kx, int& ky, int& ks) {
    kx = i / g.ny;
    ky = i - kx * g.ny;
    ks = signed_k(ky, g.ny);
}

// q = E D lW;  lN = (b10 or dt) q + E lM;  lM <- b11 q (0 after the Euler step)
__global__ void k_adj_q(AdjArgs a) {
    const int n = a.g.hx * a.g.ny;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int kx, ky, ks;
        adj_mode(a.g, i, kx, ky, ks);
        const int ka = ks < 0 ? -ks : ks;
        const bool keep = ((a.g.idealis != 1) || (ka < a.dcut[kx])) && (ky != a.g.ny / 2);
        const double E = a.etab[kx] * a.etab[a.g.hx + ka];
        const C2<double> l = a.lW[i], m = a.lM[i];
        const double ed = keep ? E : 0.0;
        const C2<double> qq = mk<double>(ed * l.x, ed * l.y);
        const double bN = a.euler ? a.dt : a.b10;
        a.q[i] = qq;
        a.lN[i] = mk<double>(bN * qq.x + E * m.x, bN * qq.y + E * m.y);
        a.lM[i] = a.euler ? mk<double>(0.0, 0.0) : mk<double>(a.b11 * qq.x, a.b11 * qq.y);
    }
}

// X0 = w lN / (nx ny), X1 = w (-i kx) lN / (nx ny), X2 = w (i ky) lN / (nx ny)
__global__ void k_adj_w3(AdjArgs a) {
    const int n = a.g.hx * a.g.ny;
    const double inv = 1.0 / ((double)a.g.nx * (double)a.g.ny);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int kx, ky, ks;
        adj_mode(a.g, i, kx, ky, ks);
        const double w = (kx == 0 ? 1.0 : 0.5) * inv;
        const C2<double> l = cscale<double>(a.lN[i], w);
        a.X0[i] = l;
        a.X1[i] = cimul<double>(l, -(double)kx * a.g.kxs);
        a.X2[i] = cimul<double>(l, (double)ks * a.g.kys);
    }
}

// physical part: nl = -(u wx + v wy), pen1 = -chi u, pen2 = -chi v
__global__ void k_adj_phys(AdjArgs a, size_t ncell) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ncell; i += (size_t)gridDim.x * blockDim.x) {
        const double ln = a.lnl[i], l1 = a.lp1[i], l2 = a.lp2[i], chi = a.mask[i];
        const double u = a.u[i], v = a.v[i];
        a.lu[i] = -a.wx[i] * ln - chi * l1;
        a.lv[i] = -a.wy[i] * ln - chi * l2;
        a.lwx[i] = -u * ln;
        a.lwy[i] = -v * ln;
        a.gmask[i] += -u * l1 - v * l2;
    }
}

// lW <- q + s (-i kx G1 - i ky G2 - i ky Pi G3 + i kx Pi G4) + c_obj Gd,  s = nx ny (1 + [kx > 0])
__global__ void k_adj_combine(AdjArgs a) {
    const int n = a.g.hx * a.g.ny;
    const double N = (double)a.g.nx * (double)a.g.ny;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int kx, ky, ks;
        adj_mode(a.g, i, kx, ky, ks);
        const double kxs = (double)kx * a.g.kxs, kys = (double)ks * a.g.kys;
        const double k2 = (double)(kx * kx) * a.g.scalex + (double)(ks * ks) * a.g.scaley;
        const double pi = (kx == 0 && ky == 0) ? 0.0 : 1.0 / k2;
        const double s = N * (kx == 0 ? 1.0 : 2.0);
        C2<double> t = cadd<double>(cimul<double>(a.G1[i], -kxs), cimul<double>(a.G2[i], -kys));
        t = cadd<double>(t, cscale<double>(cimul<double>(a.G3[i], -kys), pi));
        t = cadd<double>(t, cscale<double>(cimul<double>(a.G4[i], kxs), pi));
        const C2<double> qq = a.q[i], gd = a.Gd[i];
        a.lW[i] = mk<double>(qq.x + s * t.x + a.c_obj * gd.x, qq.y + s * t.y + a.c_obj * gd.y);
    }
}

// G3 = F(dx dy chi 1_window).  Drag = dx dy sum_window chi (u - u_s) with u = Phi(i ky Pi W) + U:
// Gd = nx ny (1 + [kx > 0]) Pi (-i ky) G3 = d drag / d W.  Lift uses v = -Phi(i kx Pi W) + V:
// Gd = nx ny (1 + [kx > 0]) Pi (i kx) G3 = d lift / d W.
__global__ void k_adj_gdrag(AdjArgs a) {
    const int n = a.g.hx * a.g.ny;
    const double N = (double)a.g.nx * (double)a.g.ny;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int kx, ky, ks;
        adj_mode(a.g, i, kx, ky, ks);
        const double kys = (double)ks * a.g.kys, kxs = (double)kx * a.g.kxs;
        const double k2 = (double)(kx * kx) * a.g.scalex + (double)(ks * ks) * a.g.scaley;
        const double pi = (kx == 0 && ky == 0) ? 0.0 : 1.0 / k2;
        const double s = N * (kx == 0 ? 1.0 : 2.0);
        a.Gd[i] = cscale<double>(cimul<double>(a.G3[i], a.comp ? kxs : -kys), s * pi);
    }
}

// per-block partial sums of |k|^2 (Wn . lW + Mn . lM): the viscosity term of one step
__global__ void __launch_bounds__(256) k_adj_nu(AdjArgs a) {
    __shared__ double sm[8];
    const int n = a.g.hx * a.g.ny;
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int kx, ky, ks;
        adj_mode(a.g, i, kx, ky, ks);
        const double k2 = (double)(kx * kx) * a.g.scalex + (double)(ks * ks) * a.g.scaley;
        const C2<double> w = a.Wn[i], lw = a.lW[i], m = a.Mn[i], lm = a.lM[i];
        s += k2 * (w.x * lw.x + w.y * lw.y + m.x * lm.x + m.y * lm.y);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
        a.part[blockIdx.x] = t;
    }
}

// acc[slot] += scale * sum(part[0 .. nparts)), in a fixed order
__global__ void k_adj_reduce(const double* part, int nparts, double scale, double* acc) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < nparts; ++i) t += part[i];
        *acc += scale * t;
    }
}

// forward sweep: ubar += c u (drag) or c v (lift), J += c Force(comp)
__global__ void k_adj_accum(AdjArgs a, size_t ncell) {
    const double* vel = a.comp ? a.v : a.u;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ncell; i += (size_t)gridDim.x * blockDim.x)
        a.ubar[i] += a.c_obj * vel[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.J += a.c_obj * a.S->force[a.comp];
}

// h = dx dy chi 1_window (physical, into lu), and the final mask gradient
// gmask += dx dy ubar 1_window (ubar: the weighted sum of u for the drag, of v for the lift)
__global__ void k_adj_window(AdjArgs a, int ix0, int ix1, int iy0, int iy1, int final_pass) {
    const int nx = a.g.nx, ny = a.g.ny;
    const double dxdy = a.g.dx * a.g.dy;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (size_t)nx * ny; i += (size_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i % nx), iy = (int)(i / nx);
        const bool in = ix >= ix0 && ix <= ix1 && iy >= iy0 && iy <= iy1;
        if (final_pass) {
            if (in) a.gmask[i] += dxdy * a.ubar[i];
        } else {
            a.lu[i] = in ? dxdy * a.mask[i] : 0.0;
        }
    }
}

}  // namespace fsibe
