// Reference elements, quadrature rules, structured meshes and DOF numbering
// for the GB300 generic-assembly backend (host side).
//
// These are the read-only inputs of the assembly hot path:
//  - Lagrange bases FEM_PK(N,K) on the reference simplex and FEM_QK(N,K) on
//    the reference cube, with GetFEM's node ordering
//    (src/getfem_fem.cc:719-781 PK_fem_, :792-826 tproduct_femi, :1010-1045 QK_fem);
//  - quadrature rules IM_TRIANGLE(k), IM_TETRAHEDRON(k), IM_GAUSS1D(k) and
//    IM_GAUSS_PARALLELEPIPED(N,k) (src/getfem_integration.cc, cubature/*.IM);
//  - getfem::regular_unit_mesh (src/getfem_regular_meshes.cc:26-80, :237-287)
//    with the same point and convex numbering;
//  - mesh_fem::enumerate_dof (src/getfem_mesh_fem.cc:320-460): first-encounter
//    numbering over elements in order and local DOFs in order, Qdim
//    consecutive DOFs per node.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "refpoly.h"

namespace gfgpu {

enum ElemKind { SIMPLEX = 0, HEX = 1 };

// A scalar Lagrange element on a reference convex: FEM_PK(dim,degree) for
// SIMPLEX, FEM_QK(dim,degree) for HEX.  degree 1 doubles as the geometric
// transformations GT_PK(dim,1) / GT_QK(dim,1).
struct RefElement {
  int dim = 0, kind = SIMPLEX, degree = 1, nb = 0;
  // node lattice coordinates: reference node = lattice / degree
  std::vector<int> lattice;  // nb x dim
  std::vector<refpoly::Poly> base;                // nb
  std::vector<std::vector<refpoly::Poly>> dbase;  // nb x dim
  RefElement() = default;
  RefElement(int dim, int kind, int degree);
  // base values (nb) and reference gradients (nb x dim, row-major) at x
  void eval(const double *x, double *val, double *grad) const;
  void node(int i, double *x) const;
};

struct Quadrature {
  std::string name;
  int dim = 0, nq = 0;
  std::vector<double> pts;  // nq x dim
  std::vector<double> w;    // nq
};

// Returns false when the name is not one of the supported rules.
bool quadrature_by_name(const std::string &name, Quadrature &q);

// Structured unit mesh, as getfem::regular_unit_mesh(m, {nx,..}, GT).
// jitter (optional): (nx+1)^dim x dim offsets in lattice order (x fastest),
// added to interior vertices only.
struct Mesh {
  int dim = 0, kind = SIMPLEX, nbpt = 0;
  int64_t n_points = 0, n_elements = 0;
  std::vector<double> points;     // n_points x dim
  std::vector<int64_t> cvpts;     // n_elements x nbpt
  std::vector<int32_t> lattice;   // n_points x dim (vertex lattice coords)
};
void regular_unit_mesh(int dim, int kind, int nx, const double *jitter, Mesh &m);

// DOF numbering of FEM_PK/FEM_QK(dim,degree) with qdim components on the
// given convexes.  Fills dofs (n_elements x nb: the first component's DOF
// of each local node, i.e. ind_scalar_basic_dof_of_element) and returns the
// number of DOFs.  degree 0 gives one DOF per element, numbered by element.
int64_t enumerate_dofs(int dim, int kind, int degree, int qdim, int64_t n_elements,
                       const int64_t *cvpts, std::vector<int64_t> &dofs);

// Reference coordinates of each DOF node (n_nodes x dim) for interpolation of
// data fields: node positions through the geometric transformation.
void dof_node_coordinates(const Mesh &m, int degree, int64_t n_dof, int qdim,
                          const std::vector<int64_t> &dofs, std::vector<double> &xyz);

}  // namespace gfgpu
