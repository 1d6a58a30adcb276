// Adjoint pieces behind ImplicitSystem::adjoint_qoi_parameter_sensitivity
// (src/systems/implicit_system.C:196-247, 474-623) for per-element coefficients.
//
// The reference perturbs each parameter p_j, re-assembles the residual
// R = K(p) u - F twice and forms dq/dp_j = dq/dp_j|_u - (dR/dp_j) . z by central
// differences (assemble_residual_derivatives, :474-514; delta_p = 1e-6 max(|p|, 1e-3)).
// K is linear in each element coefficient (k_e for Poisson, Young's modulus
// E_e for elasticity, F independent of both), so dR/dp_e = K_e(coef = 1) u_e
// exactly, and one pass over the elements gives every sensitivity:
//     dq/dp_e = - z_e^T K_e(1) u_e,
// evaluated per quadrature point from the gradients of u and z (geometry
// recomputed here, nothing stored per quadrature point):
//   Poisson:    z^T K_e(1) u = sum_q JxW grad z . grad u
//   elasticity: z^T K_e(1) u = sum_q JxW [lam div z div u + mu (dz_i/dx_k)(du_k/dx_i) + mu grad z : grad u]
// with lam, mu of Young's modulus 1.  k_region_fe builds the QoI derivative
// dq/du of q(u) = integral of u over a set of elements (the load vector of that
// set's indicator), the right-hand side of the adjoint solve K^T z = dq/du.
#include <cuda_runtime.h>

#include "assemble.cuh"
#include "df.cuh"
#include "../../include/libmesh_gb300.h"

namespace lmg {

namespace {

__device__ __forceinline__ double jac_inv(const double *X, const double *gd, int n_geo, double G[9]) {
  double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int a = 0; a < n_geo; ++a)
    for (int m = 0; m < 3; ++m) {
      const double g = gd[3 * a + m];
      J[3 * m + 0] += X[3 * a] * g;
      J[3 * m + 1] += X[3 * a + 1] * g;
      J[3 * m + 2] += X[3 * a + 2] * g;
    }
  const double c0 = J[4] * J[8] - J[5] * J[7], c1 = J[5] * J[6] - J[3] * J[8], c2 = J[3] * J[7] - J[4] * J[6];
  const double det = J[0] * c0 + J[1] * c1 + J[2] * c2;
  const double inv = 1.0 / det;
  G[0] = c0 * inv;
  G[1] = c1 * inv;
  G[2] = c2 * inv;
  G[3] = (J[2] * J[7] - J[1] * J[8]) * inv;
  G[4] = (J[0] * J[8] - J[2] * J[6]) * inv;
  G[5] = (J[1] * J[6] - J[0] * J[7]) * inv;
  G[6] = (J[1] * J[5] - J[2] * J[4]) * inv;
  G[7] = (J[2] * J[3] - J[0] * J[5]) * inv;
  G[8] = (J[0] * J[4] - J[1] * J[3]) * inv;
  return det;
}

template <int FORM, int N, int NV>
__global__ void k_vjp(VjpArgs v) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < v.n_elem;
       e += (int64_t)gridDim.x * blockDim.x) {
    double X[N * 3], U[N * NV], Z[N * NV];
    const int32_t *c = v.conn + e * N;
#pragma unroll
    for (int a = 0; a < N; ++a) {
#pragma unroll
      for (int d = 0; d < 3; ++d) X[3 * a + d] = v.xyz[3 * (int64_t)c[a] + d];
      const int64_t dof = (int64_t)v.eb[e * N + a] * NV;
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        U[a * NV + k] = v.u[dof + k];
        Z[a * NV + k] = v.z[dof + k];
      }
    }
    double lam = 0.0, mu = 0.0;
    if (FORM == LMG_ELASTICITY) {
      lam = v.nu / ((1. + v.nu) * (1. - 2. * v.nu));
      mu = 1. / (2. * (1. + v.nu));
    }
    double acc = 0.0;
    bool bad = false;
    for (int q = 0; q < v.fe.q; ++q) {
      double G[9];
      const double det = jac_inv(X, v.fe.gdphi + (int64_t)q * N * 3, N, G);
      bad |= !(det > 0.0);
      // reference gradients of u and z, then physical: du_k/dx_d = sum_m dG[m][d] * du_k/dxi_m
      double gu[NV][3], gz[NV][3];
#pragma unroll
      for (int k = 0; k < NV; ++k)
#pragma unroll
        for (int d = 0; d < 3; ++d) gu[k][d] = gz[k][d] = 0.0;
      const double *dp = v.fe.dphi + (int64_t)q * N * 3;
#pragma unroll
      for (int a = 0; a < N; ++a) {
        double g[3];
#pragma unroll
        for (int d = 0; d < 3; ++d)
          g[d] = dp[3 * a] * G[d] + dp[3 * a + 1] * G[3 + d] + dp[3 * a + 2] * G[6 + d];
#pragma unroll
        for (int k = 0; k < NV; ++k)
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            gu[k][d] += U[a * NV + k] * g[d];
            gz[k][d] += Z[a * NV + k] * g[d];
          }
      }
      const double jxw = det * v.fe.qw[q];
      double b = 0.0;
      if (FORM == LMG_POISSON) {
        b = gz[0][0] * gu[0][0] + gz[0][1] * gu[0][1] + gz[0][2] * gu[0][2];
      } else {
        const double divu = gu[0][0] + gu[1][1] + gu[2][2], divz = gz[0][0] + gz[1][1] + gz[2][2];
        double s1 = 0.0, s2 = 0.0;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            s1 += gz[i][k] * gu[k][i];
            s2 += gz[i][k] * gu[i][k];
          }
        b = lam * divz * divu + mu * (s1 + s2);
      }
      acc += jxw * b;
    }
    if (bad) {
      atomicCAS(v.status, 0, LMG_ERR_DEGENERATE);
      atomicMin(v.bad_elem, (unsigned long long)e);
    }
    v.out[e] = -acc;
  }
}

// Load vector of the indicator of the marked elements: Fe_a = sum_q JxW phi_a
// for every variable, zero for unmarked elements and for constrained dofs (the
// adjoint problem carries the primal's homogeneous Dirichlet rows, so z = 0
// there), as double-float pairs.
template <int N, int NV>
__global__ void k_region_fe(VjpArgs v) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < v.n_elem;
       e += (int64_t)gridDim.x * blockDim.x) {
    double fe[N];
#pragma unroll
    for (int a = 0; a < N; ++a) fe[a] = 0.0;
    if (v.region[e]) {
      double X[N * 3];
      const int32_t *c = v.conn + e * N;
#pragma unroll
      for (int a = 0; a < N; ++a)
#pragma unroll
        for (int d = 0; d < 3; ++d) X[3 * a + d] = v.xyz[3 * (int64_t)c[a] + d];
      for (int q = 0; q < v.fe.q; ++q) {
        double G[9];
        const double jxw = jac_inv(X, v.fe.gdphi + (int64_t)q * N * 3, N, G) * v.fe.qw[q];
        const double *ph = v.fe.phi + (int64_t)q * N;
#pragma unroll
        for (int a = 0; a < N; ++a) fe[a] += jxw * ph[a];
      }
    }
    const uint64_t mask = v.cmask[e];
#pragma unroll
    for (int a = 0; a < N; ++a) {
      const DF d = df_split(fe[a]);
#pragma unroll
      for (int k = 0; k < NV; ++k)
        v.Fe2[(e * N + a) * NV + k] = ((mask >> (k * N + a)) & 1ull) ? make_float2(0.f, 0.f) : make_float2(d.hi, d.lo);
    }
  }
}

// Coordinate sensitivities, Poisson form (introduction_ex4.C:464-536 weak form):
// with r = K(X) u - F(X) and q(u, X) = integral of u over the marked elements,
//   dq/dX = dq/dX|_u - z^T dr/dX,
// per element and quadrature point in reverse mode through detJ and J^{-1}
// (J_en = dx_e/dxi_n, G = J^{-1}, v = grad u, w = grad z, hats = G applied again):
//   d(detJ)/dJ_en          = detJ G_ne
//   d(detJ w.v)/dJ_en      = detJ (G_ne w.v - v_e w^_n - w_e v^_n)
// and dJ_en/dX_ae = dphi_map_a/dxi_n.  Every quadrature point takes its own
// Jacobian, which is what central differences of the reference's assembly see
// (a perturbed affine element is no longer affine).
template <int N>
__global__ void k_vjp_xyz(VjpArgs v) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < v.n_elem;
       e += (int64_t)gridDim.x * blockDim.x) {
    double X[N * 3], U[N], Z[N], Fn[N], dX[N * 3];
    const int32_t *c = v.conn + e * N;
#pragma unroll
    for (int a = 0; a < N; ++a) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        X[3 * a + d] = v.xyz[3 * (int64_t)c[a] + d];
        dX[3 * a + d] = 0.0;
      }
      const int64_t dof = v.eb[e * N + a];
      U[a] = v.u[dof];
      Z[a] = v.z[dof];
      Fn[a] = v.nodal_f ? v.nodal_f[c[a]] : 0.0;
    }
    const double k = v.coef ? v.coef[e] : 1.0;
    const bool in_q = v.region && v.region[e];
    bool bad = false;
    for (int q = 0; q < v.fe.q; ++q) {
      const double *gd = v.fe.gdphi + (int64_t)q * N * 3;
      double G[9];
      const double det = jac_inv(X, gd, N, G);
      bad |= !(det > 0.0);
      const double *dp = v.fe.dphi + (int64_t)q * N * 3, *ph = v.fe.phi + (int64_t)q * N;
      double gu[3] = {0, 0, 0}, gz[3] = {0, 0, 0}, uq = 0.0, zq = 0.0, fq = 0.0;
#pragma unroll
      for (int a = 0; a < N; ++a) {
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          gu[m] += dp[3 * a + m] * U[a];
          gz[m] += dp[3 * a + m] * Z[a];
        }
        uq += ph[a] * U[a];
        zq += ph[a] * Z[a];
        fq += ph[a] * Fn[a];
      }
      double vv[3], ww[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        vv[d] = G[d] * gu[0] + G[3 + d] * gu[1] + G[6 + d] * gu[2];
        ww[d] = G[d] * gz[0] + G[3 + d] * gz[1] + G[6 + d] * gz[2];
      }
      double vh[3], wh[3];
#pragma unroll
      for (int n = 0; n < 3; ++n) {
        vh[n] = G[3 * n] * vv[0] + G[3 * n + 1] * vv[1] + G[3 * n + 2] * vv[2];
        wh[n] = G[3 * n] * ww[0] + G[3 * n + 1] * ww[1] + G[3 * n + 2] * ww[2];
      }
      const double jw = det * v.fe.qw[q];
      const double dot = vv[0] * ww[0] + vv[1] * ww[1] + vv[2] * ww[2];
      // d/dJ of  (in_q ? jw uq : 0) - (k jw w.v - jw f z)
      const double scal = (in_q ? jw * uq : 0.0) - k * jw * dot + jw * fq * zq;
#pragma unroll
      for (int ee = 0; ee < 3; ++ee)
#pragma unroll
        for (int n = 0; n < 3; ++n) {
          const double cj = G[3 * n + ee] * scal + k * jw * (vv[ee] * wh[n] + ww[ee] * vh[n]);
#pragma unroll
          for (int a = 0; a < N; ++a) dX[3 * a + ee] += cj * gd[3 * a + n];
        }
    }
    if (bad) {
      atomicCAS(v.status, 0, LMG_ERR_DEGENERATE);
      atomicMin(v.bad_elem, (unsigned long long)e);
    }
#pragma unroll
    for (int i = 0; i < N * 3; ++i) v.xout[e * N * 3 + i] = dX[i];
  }
}

// Coordinate sensitivities of the elasticity form, the same reverse mode: per
// quadrature point, with P_u = grad u, P_z = grad z (3 x 3, rows = components),
//   W = lam tr P_z tr P_u + mu sum_ij P_z,ij (P_u,ij + P_u,ji)
//   S_u = dW/dP_u = lam tr P_z I + mu (P_z + P_z^T),  S_z likewise,
//   d P_u,kd / dJ_en = -G_nd P_u,ke,
// so -dW/dJ_en = sum_k (S_u G^T)_kn P_u,ke + (S_z G^T)_kn P_z,ke; the QoI is the
// integral of the sum of u's components over the marked elements and the load
// term sum_k f_k z_k (what k_region_fe and the element kernel use).
template <int N>
__global__ void k_vjp_xyz_el(VjpArgs v) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < v.n_elem;
       e += (int64_t)gridDim.x * blockDim.x) {
    double X[N * 3], dX[N * 3];
    const int32_t *c = v.conn + e * N;
#pragma unroll
    for (int a = 0; a < N; ++a)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        X[3 * a + d] = v.xyz[3 * (int64_t)c[a] + d];
        dX[3 * a + d] = 0.0;
      }
    const double E = v.coef ? v.coef[e] : 1.0;
    const double lam = (E * v.nu) / ((1. + v.nu) * (1. - 2. * v.nu)), mu = E / (2. * (1. + v.nu));
    const bool in_q = v.region && v.region[e];
    bool bad = false;
    for (int q = 0; q < v.fe.q; ++q) {
      const double *gd = v.fe.gdphi + (int64_t)q * N * 3;
      double G[9];
      const double det = jac_inv(X, gd, N, G);
      bad |= !(det > 0.0);
      const double *dp = v.fe.dphi + (int64_t)q * N * 3, *ph = v.fe.phi + (int64_t)q * N;
      double gu[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, gz[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // [k][m]
      double usum = 0.0, fz = 0.0;
      double fq[3] = {0.0, 0.0, 0.0}, zq[3] = {0.0, 0.0, 0.0};
      for (int a = 0; a < N; ++a) {
        const int64_t b3 = (int64_t)v.eb[e * N + a] * 3;
        const double pa = ph[a];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const double uk = v.u[b3 + k], zk = v.z[b3 + k];
#pragma unroll
          for (int m = 0; m < 3; ++m) {
            gu[3 * k + m] += dp[3 * a + m] * uk;
            gz[3 * k + m] += dp[3 * a + m] * zk;
          }
          usum += pa * uk;
          zq[k] += pa * zk;
          if (v.nodal_f) fq[k] += pa * v.nodal_f[3 * (int64_t)c[a] + k];
        }
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) fz += fq[k] * zq[k];
      double Pu[9], Pz[9];  // [k][d] = sum_m G[3m+d] g[k][m]
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          Pu[3 * k + d] = G[d] * gu[3 * k] + G[3 + d] * gu[3 * k + 1] + G[6 + d] * gu[3 * k + 2];
          Pz[3 * k + d] = G[d] * gz[3 * k] + G[3 + d] * gz[3 * k + 1] + G[6 + d] * gz[3 * k + 2];
        }
      const double tu = Pu[0] + Pu[4] + Pu[8], tz = Pz[0] + Pz[4] + Pz[8];
      double W = lam * tz * tu;
      double Su[9], Sz[9];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          W += mu * Pz[3 * i + j] * (Pu[3 * i + j] + Pu[3 * j + i]);
          Su[3 * i + j] = mu * (Pz[3 * i + j] + Pz[3 * j + i]) + (i == j ? lam * tz : 0.0);
          Sz[3 * i + j] = mu * (Pu[3 * i + j] + Pu[3 * j + i]) + (i == j ? lam * tu : 0.0);
        }
      const double jw = det * v.fe.qw[q];
      const double scal = (in_q ? jw * usum : 0.0) - jw * W + jw * fz;
      // SG[k][n] = sum_d S[k][d] G[3n+d]
      double SGu[9], SGz[9];
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int n = 0; n < 3; ++n) {
          SGu[3 * k + n] = Su[3 * k] * G[3 * n] + Su[3 * k + 1] * G[3 * n + 1] + Su[3 * k + 2] * G[3 * n + 2];
          SGz[3 * k + n] = Sz[3 * k] * G[3 * n] + Sz[3 * k + 1] * G[3 * n + 1] + Sz[3 * k + 2] * G[3 * n + 2];
        }
#pragma unroll
      for (int ee = 0; ee < 3; ++ee)
#pragma unroll
        for (int n = 0; n < 3; ++n) {
          double dw = 0.0;
#pragma unroll
          for (int k = 0; k < 3; ++k) dw += SGu[3 * k + n] * Pu[3 * k + ee] + SGz[3 * k + n] * Pz[3 * k + ee];
          const double cj = G[3 * n + ee] * scal + jw * dw;
#pragma unroll
          for (int a = 0; a < N; ++a) dX[3 * a + ee] += cj * gd[3 * a + n];
        }
    }
    if (bad) {
      atomicCAS(v.status, 0, LMG_ERR_DEGENERATE);
      atomicMin(v.bad_elem, (unsigned long long)e);
    }
#pragma unroll
    for (int i = 0; i < N * 3; ++i) v.xout[e * N * 3 + i] = dX[i];
  }
}

// Per-dof sums of the element node contributions, in element order.
__global__ void k_gather_xyz(VjpArgs v) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < v.n_rows;
       r += (int64_t)gridDim.x * blockDim.x) {
    double s[3] = {0.0, 0.0, 0.0};
    for (int32_t t = v.fptr[r]; t < v.fptr[r + 1]; ++t) {
      const int64_t code = v.fcontrib[t];
#pragma unroll
      for (int d = 0; d < 3; ++d) s[d] += v.xout[code * 3 + d];
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) v.row_out[r * 3 + d] = s[d];
  }
}

template <int FORM, int N, int NV>
void launch_v(bool region, const VjpArgs &v, int grid, cudaStream_t s) {
  const int64_t blocks = (v.n_elem + 127) / 128;
  const int g = (int)(blocks < grid ? blocks : grid);
  if (region) k_region_fe<N, NV><<<g, 128, 0, s>>>(v);
  else k_vjp<FORM, N, NV><<<g, 128, 0, s>>>(v);
}

}  // namespace

bool launch_vjp_xyz(int form, int n, const VjpArgs &v, int grid, cudaStream_t s) {
  const int64_t blocks = (v.n_elem + 127) / 128;
  const int g = (int)(blocks < grid ? blocks : grid);
  if (form == LMG_ELASTICITY) {
    if (n == 4) k_vjp_xyz_el<4><<<g, 128, 0, s>>>(v);
    else if (n == 6) k_vjp_xyz_el<6><<<g, 128, 0, s>>>(v);
    else if (n == 8) k_vjp_xyz_el<8><<<g, 128, 0, s>>>(v);
    else if (n == 10) k_vjp_xyz_el<10><<<g, 128, 0, s>>>(v);
    else return false;
  } else if (n == 4) k_vjp_xyz<4><<<g, 128, 0, s>>>(v);
  else if (n == 6) k_vjp_xyz<6><<<g, 128, 0, s>>>(v);
  else if (n == 8) k_vjp_xyz<8><<<g, 128, 0, s>>>(v);
  else if (n == 10) k_vjp_xyz<10><<<g, 128, 0, s>>>(v);
  else if (n == 27) k_vjp_xyz<27><<<g, 128, 0, s>>>(v);
  else return false;
  const int64_t rb = (v.n_rows + 255) / 256;
  k_gather_xyz<<<(int)(rb < grid ? rb : grid), 256, 0, s>>>(v);
  return true;
}

bool launch_vjp(int form, int n, int nv, bool region, const VjpArgs &v, int grid, cudaStream_t s) {
#define LMG_V(F, NN, V)                          \
  if (form == F && n == NN && nv == V) {         \
    launch_v<F, NN, V>(region, v, grid, s);      \
    return true;                                 \
  }
  LMG_V(LMG_POISSON, 4, 1)
  LMG_V(LMG_POISSON, 6, 1)
  LMG_V(LMG_POISSON, 8, 1)
  LMG_V(LMG_POISSON, 10, 1)
  LMG_V(LMG_POISSON, 27, 1)
  LMG_V(LMG_ELASTICITY, 4, 3)
  LMG_V(LMG_ELASTICITY, 6, 3)
  LMG_V(LMG_ELASTICITY, 8, 3)
  LMG_V(LMG_ELASTICITY, 10, 3)
#undef LMG_V
  return false;
}

}  // namespace lmg
