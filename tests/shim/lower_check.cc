// Test program (CPU): lowers GWFL expressions with the C++ lowering of the
// GetFEM-side drop-in (getfem_gb300/getfem_shim/gfgpu_lower.cc), walking the
// trees that the reference's own ga_workspace::add_expression analysed and
// derived, and prints one JSON line per case and order.
//
// Input (standard input), one case per line, fields separated by '|':
//   name|dim|nx|gt|degree|qdim|im|expr|data
// data: comma-separated name:KIND with KIND P0 (per element), S (scalar
// field on the variable's fem), V (field on the variable's mesh_fem), or
// C=v1;v2;... (fixed-size constant with those values).
// Output: {"name": ..., "order": o, "forms": [...]} or {..., "error": "..."}.
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "getfem/getfem_generic_assembly.h"
#include "getfem/getfem_mesh_fem.h"
#include "getfem/getfem_mesh_im.h"
#include "getfem/getfem_regular_meshes.h"
#include "gfgpu_getfem.h"

static std::vector<std::string> split(const std::string &s, char c) {
  std::vector<std::string> out;
  std::string cur;
  for (char ch : s) {
    if (ch == c) {
      out.push_back(cur);
      cur.clear();
    } else {
      cur += ch;
    }
  }
  out.push_back(cur);
  return out;
}

static std::string esc(const std::string &s) {
  std::string o;
  for (char c : s) {
    if (c == '"' || c == '\\') o += '\\';
    if (c == '\n') { o += "\\n"; continue; }
    o += c;
  }
  return o;
}

int main() {
  std::string line;
  while (std::getline(std::cin, line)) {
    if (line.empty() || line[0] == '#') continue;
    auto f = split(line, '|');
    if (f.size() != 9) {
      std::cerr << "bad line: " << line << "\n";
      return 2;
    }
    const std::string name = f[0], gt = f[3], im = f[6], expr = f[7];
    const int dim = std::stoi(f[1]), nx = std::stoi(f[2]), deg = std::stoi(f[4]),
              qdim = std::stoi(f[5]);
    char buf[128];
    std::snprintf(buf, sizeof buf, "GT_%s(%d,1)", gt.c_str(), dim);
    getfem::mesh m;
    std::vector<bgeot::size_type> ns(dim, bgeot::size_type(nx));
    getfem::regular_unit_mesh(m, ns, bgeot::geometric_trans_descriptor(buf));
    std::snprintf(buf, sizeof buf, "FEM_%s(%d,%d)", gt.c_str(), dim, deg);
    getfem::pfem pf = getfem::fem_descriptor(buf);
    std::snprintf(buf, sizeof buf, "FEM_%s(%d,0)", gt.c_str(), dim);
    getfem::pfem pf0 = getfem::fem_descriptor(buf);
    getfem::mesh_fem mf(m, bgeot::dim_type(qdim)), mfs(m, 1), mf0(m, 1);
    mf.set_finite_element(m.convex_index(), pf);
    mfs.set_finite_element(m.convex_index(), pf);
    mf0.set_finite_element(m.convex_index(), pf0);
    getfem::mesh_im mim(m);
    mim.set_integration_method(m.convex_index(), getfem::int_method_descriptor(im));
    std::vector<std::vector<double>> store;
    store.reserve(16);
    getfem::ga_workspace ws;
    store.emplace_back(mf.nb_dof(), 0.1);
    ws.add_fem_variable("u", mf, gmm::sub_interval(0, mf.nb_dof()), store.back());
    std::string err;
    try {
      for (const std::string &d : split(f[8], ',')) {
        if (d.empty()) continue;
        auto kv = split(d, ':');
        const std::string &nm = kv[0], &k = kv[1];
        if (k == "P0") {
          store.emplace_back(mf0.nb_dof(), 1.0);
          ws.add_fem_constant(nm, mf0, store.back());
        } else if (k == "S") {
          store.emplace_back(mfs.nb_dof(), 1.0);
          ws.add_fem_constant(nm, mfs, store.back());
        } else if (k == "V") {
          store.emplace_back(mf.nb_dof(), 1.0);
          ws.add_fem_constant(nm, mf, store.back());
        } else if (k.size() > 2 && k[0] == 'C' && k[1] == '=') {
          std::vector<double> v;
          for (const std::string &x : split(k.substr(2), ';')) v.push_back(std::stod(x));
          store.push_back(v);
          ws.add_fixed_size_constant(nm, store.back());
        }
      }
      ws.add_expression(expr, mim);
    } catch (const std::exception &e) {
      err = e.what();
    }
    for (size_t order = 0; order <= 2; ++order) {
      std::cout << "{\"name\": \"" << esc(name) << "\", \"order\": " << order;
      if (!err.empty()) {
        std::cout << ", \"error\": \"add_expression: " << esc(err) << "\"}\n";
        continue;
      }
      try {
        auto forms = gfgpu_getfem::lower_workspace(ws, order);
        std::cout << ", \"forms\": [";
        for (size_t i = 0; i < forms.size(); ++i)
          std::cout << (i ? ", " : "") << gfgpu_getfem::to_json(forms[i]);
        std::cout << "]}\n";
      } catch (const std::exception &e) {
        std::cout << ", \"error\": \"" << esc(e.what()) << "\"}\n";
      }
    }
  }
  return 0;
}
