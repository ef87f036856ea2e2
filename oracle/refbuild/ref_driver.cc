// Fixture and timing driver for the reference GetFEM build (test
// infrastructure only).  It runs the reference's own generic assembly
// (ga_workspace::add_expression + ga_workspace::assembly, see
// src/getfem_generic_assembly_workspace.cc:545 and :791) on a structured
// unit mesh built by getfem::regular_unit_mesh
// (src/getfem_regular_meshes.cc:237), with input vectors read from files,
// and dumps the mesh, the DOF maps and the assembled K (as CSR), R and
// potential as raw little-endian binaries.
//
// usage: ref_driver key=value ...
//   dim=2|3 nx=N gt=PK|QK fem=K qdim=Q im=IM_NAME in=DIR out=DIR
//   expr=GWFL  orders=2,1,0  reps=R  jitter=0|1
//   solve=cg resmax=R maxiter=N   (after the orders: solve K x = -R with
//       homogeneous Dirichlet conditions on the boundary DOFs eliminated as
//       the model's dof constraints do, getfem_models.cc:2806-2870, by
//       gmm::cg with the identity preconditioner; writes x.bin and the
//       iteration count)
//   consts=name:KIND,...   KIND = P0 (one value per element),
//                                 S  (scalar field on the same FEM),
//                                 V  (field on the variable's FEM, qdim Q),
//                                 C  (fixed-size constant, file length)
//   internal=NAME expr2=GWFL   (condensation case: the variables live in a
//       getfem::model, u plus the internal im_data variable NAME, scalar per
//       Gauss point, values in/NAME.bin; both expressions are added to a
//       ga_workspace over the model; the driver runs assembly(1, true) and
//       writes R_full.bin (primary + internal rows), then, with that residual
//       as the assembled vector, assembly(2, true) and writes the condensed K
//       (K_*.bin), the vector Rc.bin and the internal coupling matrix
//       (C_rowptr/C_colidx/C_vals.bin), workspace.cc:791-860)
//   time=model threads=T warmup=W steps=S   (timing of the reference's
//       multi-threaded assembly: u a variable of a getfem::model, the data
//       initialized fem data, the expression a nonlinear term brick
//       (getfem::add_nonlinear_term, re-assembled at every call), and
//       model::assembly(BUILD_ALL) (K and the right-hand side,
//       src/getfem_models.cc:2646-2730: one ga_workspace per OpenMP thread
//       over that thread's partition of the region) run W + S times with T
//       threads; writes the S step times, nnz(K) and the norms of K and of
//       the right-hand side to info.json; model_out=1 also writes the
//       tangent matrix K_*.bin and rhs.bin)
//   dump=0   (skip the mesh / DOF map / reference-element dumps)
//   vars=name:KIND,...   (data declared as variables after u, KIND as for
//       consts but P0 / S / V only: the order-1 vector of a potential then
//       holds dE/d(name) after the u rows)
// The variable is always "u" (file in/u.bin, zeros when absent).
// Jitter: when jitter=1, in/jitter.bin holds (nx+1)^dim x dim doubles in
// lattice order (x index fastest); interior vertices are moved by it.
#include "getfem/getfem_generic_assembly.h"
#include "getfem/getfem_models.h"
#include "getfem/getfem_omp.h"
#include "getfem/getfem_im_data.h"
#include "getfem/getfem_regular_meshes.h"
#include "getfem/getfem_mesh_fem.h"
#include "getfem/getfem_mesh_im.h"
#include "gmm/gmm_solver_cg.h"
#include <chrono>
#include <cstdio>
#include <fstream>
#include <map>
#include <algorithm>
#include <cmath>

using bgeot::size_type;
using bgeot::scalar_type;

static std::map<std::string, std::string> args;

static std::string arg(const std::string &k, const std::string &d = "") {
  auto it = args.find(k);
  return it == args.end() ? d : it->second;
}

static bool read_file(const std::string &path, std::vector<double> &v) {
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  if (!f) return false;
  std::streamsize n = f.tellg();
  f.seekg(0);
  v.resize(size_t(n) / sizeof(double));
  f.read(reinterpret_cast<char *>(v.data()), n);
  return true;
}

template <typename T>
static void write_file(const std::string &path, const std::vector<T> &v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(T));
}

static std::vector<std::string> split(const std::string &s, char c) {
  std::vector<std::string> out;
  std::string cur;
  for (char ch : s) {
    if (ch == c) { out.push_back(cur); cur.clear(); }
    else cur += ch;
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

// column-major sparse matrix -> CSR files (rows sorted, columns ascending)
template <typename MAT>
static int64_t write_csr(const std::string &prefix, const MAT &K) {
  size_type n = gmm::mat_nrows(K);
  std::vector<int64_t> rowptr(n + 1, 0);
  for (size_type j = 0; j < gmm::mat_ncols(K); ++j)
    for (const auto &e : K.col(j)) rowptr[e.c + 1]++;
  for (size_type i = 0; i < n; ++i) rowptr[i + 1] += rowptr[i];
  std::vector<int64_t> colidx(rowptr[n]), fill(rowptr.begin(), rowptr.end() - 1);
  std::vector<double> vals(rowptr[n]);
  for (size_type j = 0; j < gmm::mat_ncols(K); ++j)
    for (const auto &e : K.col(j)) {
      int64_t k = fill[e.c]++;
      colidx[k] = int64_t(j);
      vals[k] = e.e;
    }
  write_file(prefix + "_rowptr.bin", rowptr);
  write_file(prefix + "_colidx.bin", colidx);
  write_file(prefix + "_vals.bin", vals);
  return rowptr[n];
}

static double median(std::vector<double> v) {
  if (v.empty()) return 0;
  std::sort(v.begin(), v.end());
  return v[v.size() / 2];
}

int main(int argc, char **argv) {
  for (int i = 1; i < argc; ++i) {
    std::string a(argv[i]);
    size_t p = a.find('=');
    if (p != std::string::npos) args[a.substr(0, p)] = a.substr(p + 1);
  }
  // the thread count is fixed before any GetFEM object exists: the
  // per-thread storage of GetFEM's singletons is sized at creation
  const int threads = std::stoi(arg("threads", "1"));
  getfem::set_num_threads(threads);
  if (arg("time", "") == "model") gmm::set_traces_level(0);
  int dim = std::stoi(arg("dim", "2"));
  size_type nx = std::stoul(arg("nx", "4"));
  std::string gt = arg("gt", "PK");
  int deg = std::stoi(arg("fem", "1"));
  int qdim = std::stoi(arg("qdim", "1"));
  std::string imname = arg("im", "IM_TRIANGLE(2)");
  std::string in = arg("in", "."), out = arg("out", ".");
  std::string expr = arg("expr", "Grad_u.Grad_Test_u");
  int reps = std::stoi(arg("reps", "1"));
  bool jitter = arg("jitter", "0") == "1";

  char buf[128];
  snprintf(buf, sizeof buf, "GT_%s(%d,1)", gt.c_str(), dim);
  bgeot::pgeometric_trans pgt = bgeot::geometric_trans_descriptor(buf);
  getfem::mesh m;
  std::vector<size_type> nsubdiv(dim, nx);
  getfem::regular_unit_mesh(m, nsubdiv, pgt);

  if (jitter) {
    std::vector<double> J;
    if (!read_file(in + "/jitter.bin", J)) { fprintf(stderr, "no jitter.bin\n"); return 2; }
    for (dal::bv_visitor ip(m.points().index()); !ip.finished(); ++ip) {
      bgeot::base_node &P = m.points()[ip];
      size_type flat = 0, stride = 1;
      bool interior = true;
      for (int d = 0; d < dim; ++d) {
        long l = lround(P[d] * double(nx));
        if (l <= 0 || l >= long(nx)) interior = false;
        flat += size_type(l) * stride;
        stride *= (nx + 1);
      }
      if (interior)
        for (int d = 0; d < dim; ++d) P[d] += J[flat * dim + d];
    }
  }

  snprintf(buf, sizeof buf, "FEM_%s(%d,%d)", gt.c_str(), dim, deg);
  getfem::pfem pf = getfem::fem_descriptor(buf);
  snprintf(buf, sizeof buf, "FEM_%s(%d,0)", gt.c_str(), dim);
  getfem::pfem pf0 = getfem::fem_descriptor(buf);

  getfem::mesh_fem mf(m, bgeot::dim_type(qdim));
  mf.set_finite_element(m.convex_index(), pf);
  getfem::mesh_fem mfs(m, 1);
  mfs.set_finite_element(m.convex_index(), pf);
  getfem::mesh_fem mf0(m, 1);
  mf0.set_finite_element(m.convex_index(), pf0);
  getfem::mesh_im mim(m);
  mim.set_integration_method(m.convex_index(), getfem::int_method_descriptor(imname));

  size_type ndof = mf.nb_dof();
  size_type E = m.nb_convex();

  const bool dump = arg("dump", "1") != "0";
  // reference-element tables: integration points, weights, and the FEM's
  // base values / reference gradients at those points
  if (dump) {
    getfem::pintegration_method pim = getfem::int_method_descriptor(imname);
    const getfem::papprox_integration pai = pim->approx_method();
    std::vector<double> ipts, iw, bval, bgrad;
    size_type nq = pai->nb_points_on_convex();
    for (size_type q = 0; q < nq; ++q) {
      for (int d = 0; d < dim; ++d) ipts.push_back(pai->point(q)[d]);
      iw.push_back(pai->coeff(q));
      getfem::base_tensor t;
      pf->base_value(pai->point(q), t);
      for (size_type k = 0; k < t.size(); ++k) bval.push_back(t[k]);
      pf->grad_base_value(pai->point(q), t);
      for (size_type k = 0; k < t.size(); ++k) bgrad.push_back(t[k]);
    }
    write_file(out + "/im_points.bin", ipts);
    write_file(out + "/im_weights.bin", iw);
    write_file(out + "/base_val.bin", bval);
    write_file(out + "/base_grad.bin", bgrad);
    std::vector<double> nodes;
    for (size_type i = 0; i < pf->nb_dof(0); ++i)
      for (int d = 0; d < dim; ++d) nodes.push_back(pf->node_of_dof(0, i)[d]);
    write_file(out + "/fem_nodes.bin", nodes);
  }

  // mesh and DOF maps
  if (dump) {
    std::vector<double> pts;
    for (size_type ip = 0; ip < m.points().size(); ++ip)
      for (int d = 0; d < dim; ++d) pts.push_back(m.points()[ip][d]);
    write_file(out + "/points.bin", pts);
    std::vector<int64_t> cvp, dofs, dofs0;
    for (size_type cv = 0; cv < E; ++cv) {
      for (size_type p : m.ind_points_of_convex(cv)) cvp.push_back(int64_t(p));
      for (size_type d : mf.ind_scalar_basic_dof_of_element(cv)) dofs.push_back(int64_t(d));
      { auto ct0 = mf0.ind_basic_dof_of_element(cv); for (size_type d : ct0) dofs0.push_back(int64_t(d)); }
    }
    write_file(out + "/cvpts.bin", cvp);
    write_file(out + "/dofs.bin", dofs);
    write_file(out + "/dofs0.bin", dofs0);
  }

  getfem::ga_workspace ws;
  std::vector<double> U(ndof, 0.0);
  read_file(in + "/u.bin", U);
  if (U.size() != ndof) { fprintf(stderr, "u.bin has %zu values, need %zu\n", U.size(), size_t(ndof)); return 2; }

  if (arg("time", "") == "model") {
    getfem::model md;
    md.add_fem_variable("u", mf);
    gmm::copy(U, md.set_real_variable("u"));
    for (const std::string &c : split(arg("consts", ""), ',')) {
      std::vector<std::string> kv = split(c, ':');
      std::vector<double> v;
      if (!read_file(in + "/" + kv[0] + ".bin", v)) { fprintf(stderr, "missing %s\n", kv[0].c_str()); return 2; }
      const std::string &k = kv[1];
      if (k == "P0") md.add_initialized_fem_data(kv[0], mf0, v);
      else if (k == "S") md.add_initialized_fem_data(kv[0], mfs, v);
      else if (k == "V") md.add_initialized_fem_data(kv[0], mf, v);
      else md.add_initialized_fixed_size_data(kv[0], v);
    }
    getfem::add_nonlinear_term(md, mim, expr);
    const int warm = std::stoi(arg("warmup", "1")), steps = std::stoi(arg("steps", "3"));
    std::vector<double> times;
    for (int r = 0; r < warm + steps; ++r) {
      auto t0 = std::chrono::steady_clock::now();
      md.assembly(getfem::model::BUILD_ALL);
      auto t1 = std::chrono::steady_clock::now();
      if (r >= warm) times.push_back(std::chrono::duration<double>(t1 - t0).count());
    }
    const auto &K = md.real_tangent_matrix();
    if (arg("model_out", "0") == "1") {
      // the model's tangent matrix and right-hand side (rhs = -residual)
      write_csr(out + "/K", K);
      std::vector<double> rhs(md.real_rhs().begin(), md.real_rhs().end());
      write_file(out + "/rhs.bin", rhs);
    }
    size_type nnz = 0;
    double knorm = 0.0;
    for (size_type j = 0; j < gmm::mat_ncols(K); ++j)
      for (const auto &e : K.col(j)) { ++nnz; knorm += e.e * e.e; }
    const auto &rhs = md.real_rhs();
    FILE *info = fopen((out + "/info.json").c_str(), "w");
    fprintf(info, "{\"n_dof\": %zu, \"n_elements\": %zu, \"threads\": %d, \"nnz\": %zu, "
            "\"K_frobenius\": %.17g, \"rhs_norm\": %.17g, \"t_steps\": [",
            size_t(ndof), size_t(E), threads, size_t(nnz), std::sqrt(knorm), gmm::vect_norm2(rhs));
    for (size_t i = 0; i < times.size(); ++i) fprintf(info, "%s%.6e", i ? ", " : "", times[i]);
    fprintf(info, "]}\n");
    fclose(info);
    return 0;
  }

  const std::string internal = arg("internal", "");
  if (!internal.empty()) {
    getfem::model md;
    md.add_fem_variable("u", mf);
    gmm::copy(U, md.set_real_variable("u"));
    getfem::im_data imd(mim);
    md.add_internal_im_variable(internal, imd);
    std::vector<double> Pv;
    if (!read_file(in + "/" + internal + ".bin", Pv) ||
        Pv.size() != gmm::vect_size(md.real_variable(internal))) {
      fprintf(stderr, "%s.bin missing or of wrong size\n", internal.c_str());
      return 2;
    }
    gmm::copy(Pv, md.set_real_variable(internal));
    for (const std::string &c : split(arg("consts", ""), ',')) {
      std::vector<std::string> kv = split(c, ':');
      std::vector<double> v;
      if (!read_file(in + "/" + kv[0] + ".bin", v)) { fprintf(stderr, "missing %s\n", kv[0].c_str()); return 2; }
      const std::string &k = kv[1];
      if (k == "P0") md.add_initialized_fem_data(kv[0], mf0, v);
      else if (k == "S") md.add_initialized_fem_data(kv[0], mfs, v);
      else if (k == "V") md.add_initialized_fem_data(kv[0], mf, v);
      else md.add_initialized_fixed_size_data(kv[0], v);
    }
    getfem::ga_workspace wsm(md);
    wsm.add_expression(expr, mim);
    const std::string expr2 = arg("expr2", "");
    if (!expr2.empty()) wsm.add_expression(expr2, mim);
    const size_type nprim = wsm.nb_primary_dof(), nint = wsm.nb_internal_dof();
    std::vector<double> R(nprim + nint, 0.0);
    wsm.set_assembled_vector(R);
    wsm.assembly(1, true);
    write_file(out + "/R_full.bin", R);
    // the condensation reads the current residual from the assembled vector
    std::vector<double> R1(R);
    getfem::model_real_sparse_matrix K(nprim, nprim), KQ(nprim + nint, nprim);
    wsm.set_assembled_vector(R1);
    wsm.set_assembled_matrix(K);
    wsm.set_internal_coupling_matrix(KQ);
    wsm.assembly(2, true);
    int64_t nnz = write_csr(out + "/K", K);
    write_file(out + "/Rc.bin", R1);
    int64_t cnnz = write_csr(out + "/C", KQ);
    FILE *info = fopen((out + "/info.json").c_str(), "w");
    fprintf(info, "{\"n_dof\": %zu, \"n_elements\": %zu, \"n_points\": %zu, \"n_internal\": %zu, "
            "\"nnz\": %lld, \"coupling_nnz\": %lld}\n", size_t(ndof), size_t(E),
            size_t(m.points().size()), size_t(nint), (long long)nnz, (long long)cnnz);
    fclose(info);
    return 0;
  }
  ws.add_fem_variable("u", mf, gmm::sub_interval(0, ndof), U);
  std::map<std::string, std::vector<double>> cst;
  for (const std::string &c : split(arg("consts", ""), ',')) {
    std::vector<std::string> kv = split(c, ':');
    std::vector<double> &v = cst[kv[0]];
    if (!read_file(in + "/" + kv[0] + ".bin", v)) { fprintf(stderr, "missing %s\n", kv[0].c_str()); return 2; }
    const std::string &k = kv[1];
    size_type need = k == "P0" ? mf0.nb_dof() : k == "S" ? mfs.nb_dof() : k == "V" ? ndof : v.size();
    if (v.size() != need) { fprintf(stderr, "%s has %zu values, need %zu\n", kv[0].c_str(), v.size(), size_t(need)); return 2; }
    if (k == "P0") ws.add_fem_constant(kv[0], mf0, v);
    else if (k == "S") ws.add_fem_constant(kv[0], mfs, v);
    else if (k == "V") ws.add_fem_constant(kv[0], mf, v);
    else ws.add_fixed_size_constant(kv[0], v);
  }
  // data declared as variables (vars=name:P0|S|V,...), placed after u in
  // the order given: the order-1 assembly of a potential then holds its
  // derivative in each of them too (the derivative loop of add_tree,
  // workspace.cc:520-535, GWFL's Diff), in R.bin after the n_dof u rows
  size_type voff = ndof;
  for (const std::string &c : split(arg("vars", ""), ',')) {
    std::vector<std::string> kv = split(c, ':');
    std::vector<double> &v = cst[kv[0]];
    if (!read_file(in + "/" + kv[0] + ".bin", v)) { fprintf(stderr, "missing %s\n", kv[0].c_str()); return 2; }
    const std::string &k = kv[1];
    const getfem::mesh_fem &vmf = k == "P0" ? mf0 : k == "S" ? mfs : mf;
    if (v.size() != vmf.nb_dof()) { fprintf(stderr, "%s has %zu values, need %zu\n", kv[0].c_str(), v.size(), size_t(vmf.nb_dof())); return 2; }
    ws.add_fem_variable(kv[0], vmf, gmm::sub_interval(voff, v.size()), v);
    voff += v.size();
  }
  ws.add_expression(expr, mim);

  FILE *info = fopen((out + "/info.json").c_str(), "w");
  fprintf(info, "{\"n_dof\": %zu, \"n_elements\": %zu, \"n_points\": %zu", size_t(ndof), size_t(E), size_t(m.points().size()));

  for (const std::string &o : split(arg("orders", "2,1"), ',')) {
    int order = std::stoi(o);
    std::vector<double> times;
    for (int r = 0; r < std::max(reps, 1); ++r) {
      if (order == 1) {
        ws.assembled_vector().clear();
      }
      auto t0 = std::chrono::steady_clock::now();
      ws.assembly(size_type(order));
      auto t1 = std::chrono::steady_clock::now();
      times.push_back(std::chrono::duration<double>(t1 - t0).count());
    }
    fprintf(info, ", \"t_order%d\": %.6e", order, median(times));
    if (order == 2) {
      const auto &K = ws.assembled_matrix();
      size_type n = gmm::mat_nrows(K);
      // column-major rsvector -> CSR (rows sorted, columns ascending)
      std::vector<int64_t> rowptr(n + 1, 0);
      for (size_type j = 0; j < gmm::mat_ncols(K); ++j)
        for (const auto &e : K.col(j)) rowptr[e.c + 1]++;
      for (size_type i = 0; i < n; ++i) rowptr[i + 1] += rowptr[i];
      std::vector<int64_t> colidx(rowptr[n]), fill(rowptr.begin(), rowptr.end() - 1);
      std::vector<double> vals(rowptr[n]);
      for (size_type j = 0; j < gmm::mat_ncols(K); ++j)
        for (const auto &e : K.col(j)) {
          int64_t k = fill[e.c]++;
          colidx[k] = int64_t(j);
          vals[k] = e.e;
        }
      write_file(out + "/K_rowptr.bin", rowptr);
      write_file(out + "/K_colidx.bin", colidx);
      write_file(out + "/K_vals.bin", vals);
      fprintf(info, ", \"nnz\": %lld", (long long)rowptr[n]);
    } else if (order == 1) {
      write_file(out + "/R.bin", ws.assembled_vector());
    } else {
      std::vector<double> e(1, ws.assembled_potential());
      write_file(out + "/E.bin", e);
    }
  }
  if (arg("solve", "") == "cg") {
    // boundary DOFs (outer faces of the mesh)
    getfem::mesh_region border;
    getfem::outer_faces_of_mesh(m, border);
    m.region(1).clear();
    for (getfem::mr_visitor i(border); !i.finished(); ++i) m.region(1).add(i.cv(), i.f());
    dal::bit_vector bd = mf.dof_on_region(m.region(1));
    ws.assembly(2);
    ws.assembled_vector().clear();
    ws.assembly(1);
    size_type n = ndof;
    gmm::col_matrix<gmm::wsvector<double>> A(n, n);
    gmm::copy(ws.assembled_matrix(), A);
    std::vector<double> b(n), x(n, 0.0);
    gmm::copy(gmm::scaled(ws.assembled_vector(), -1.0), b);
    std::vector<bool> isd(n, false);
    for (dal::bv_visitor i(bd); !i.finished(); ++i) isd[i] = true;
    for (size_type j = 0; j < n; ++j) {
      if (isd[j]) { A.col(j).clear(); continue; }
      std::vector<size_type> rm;
      for (const auto &e : A.col(j)) if (isd[e.first]) rm.push_back(e.first);
      for (size_type i : rm) A(i, j) = 0.0;
    }
    for (size_type i = 0; i < n; ++i) if (isd[i]) { A(i, i) = 1.0; b[i] = 0.0; }
    gmm::csr_matrix<double> Acsr;
    gmm::copy(A, Acsr);
    gmm::iteration iter(std::stod(arg("resmax", "1e-12")), 0, size_t(std::stoll(arg("maxiter", "100000"))));
    auto t0 = std::chrono::steady_clock::now();
    gmm::cg(Acsr, x, b, gmm::identity_matrix(), iter);
    auto t1 = std::chrono::steady_clock::now();
    write_file(out + "/x.bin", x);
    std::vector<int64_t> bdl;
    for (dal::bv_visitor i(bd); !i.finished(); ++i) bdl.push_back(int64_t(i));
    write_file(out + "/dirichlet.bin", bdl);
    fprintf(info, ", \"cg_iterations\": %zu, \"t_cg\": %.6e", size_t(iter.get_iteration()),
            std::chrono::duration<double>(t1 - t0).count());
  }
  fprintf(info, "}\n");
  fclose(info);
  return 0;
}
