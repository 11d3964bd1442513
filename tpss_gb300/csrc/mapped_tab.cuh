// mapped_tab.cuh -- 1-D tables of the mapped SIPG operator (mapped.cu: assembly and block-sparse
// product; mapped_mf.cu: matrix-free face couplings) and the per-face geometry record.
#pragma once

namespace tpss
{
constexpr int kMapMaxNp = 8;  // k + 1 <= 8

// Lagrange basis of the cell DoFs (k + 1 nodes) at the k + 1 Gauss points and at the two faces
struct MapTab
{
  double qx[kMapMaxNp], qw[kMapMaxNp];
  double V[kMapMaxNp * kMapMaxNp], D[kMapMaxNp * kMapMaxNp];  // [i * np + q]: value, derivative
  double F[2 * kMapMaxNp], G[2 * kMapMaxNp];                  // [side * np + i]: value, derivative
};

MapTab make_tab(int k);

// Face geometry record of (cell, face f = 2 d + side), nfq = (k+1)^(dim-1) points in the order
// of the tangential Gauss indices (lowest direction fastest): [w_q][J_c^-1 n at q][J_nb^-1 n at
// q][sigma], w_q = Gauss weights * |det J| * |J^-T e_d| (surface measure), n the outer unit normal
// of the cell, J_c / J_nb the Jacobians of the cell and of the neighbour at the point
__host__ __device__ constexpr int face_geo_size(int dim, int nfq) { return nfq * (1 + 2 * dim) + 1; }
}  // namespace tpss
