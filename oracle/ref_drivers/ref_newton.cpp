// Golden-vector driver over the reference's own serial Newton path.
//
// Test infrastructure only (built by oracle/Makefile.ref into oracle/_ref/).
// It reads a line-oriented problem description, builds it with the
// reference's public API -- Space_spheric (include/spheric.hpp:1196),
// Scalar/Vector, Metric_flat::set_system, System_of_eqs::add_var/add_cst/
// add_def/add_eq_* (include/system_of_eqs.hpp:229-790) -- and writes raw
// little-endian float64 dumps of what the reference computes:
//   residual   System_of_eqs::sec_member()  (src/System_of_eqs/solver.cpp:49)
//   cols       System_of_eqs::do_col_J(c)    (solver.cpp:120)
//   jx         System_of_eqs::do_JX(x)       (solver.cpp:87)
//   fields     every unknown's coefficients, domain by domain
//   newton     do_newton_seq (src_par/do_newton.cpp:519) until converged,
//              the fields after every update and the pre-step errors.
//
// Input lines (tokens split by blanks; a string argument follows a '|'):
//   space NR NT NP NB b_1 .. b_NB        Space_spheric, CHEB_TYPE, centre 0
//   system DMIN DMAX
//   metric_flat NAME
//   scalar NAME BASE SRC                 BASE: std anti xcart ycart zcart;
//                                        SRC: a number, or a file of the values at
//                                        the collocation points, domain by domain
//   scalar_c NAME BASE FILE              a scalar given by its coefficients, domain by domain
//   vector NAME SRC                      Cartesian contravariant vector, std_base;
//                                        SRC as above, components x, y, z in turn
//   var NAME | cst NAME | cstd NAME VALUE
//   def | STRING          defd D | STRING
//   inside D | STRING     bc D B | STRING     matching D B | STRING
//   full D | STRING       firstint DMIN DMAX | INTEG | CONST
//   dump_residual FILE    dump_fields FILE    dump_jx XFILE FILE
//   dump_cols FILE C_1 C_2 ...
//   dump_coefs NAME FILE                 Base_spectral::coef of a tensor (src/Coef/coef.cpp:96)
//   dump_conf NAME FILE                  Base_spectral::coef_i of a tensor (src/Coef/coef_i.cpp:96)
//   newton PRECISION MAXSTEPS PREFIX     writes PREFIX_errors.bin and PREFIX_step<k>.bin
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "kadath.hpp"

using namespace Kadath;

namespace {

[[noreturn]] void die(const std::string& m) {
  std::cerr << "ref_newton: " << m << std::endl;
  std::exit(2);
}

std::vector<double> read_doubles(const std::string& file) {
  std::ifstream in(file, std::ios::binary);
  if (!in) die("cannot open " + file);
  in.seekg(0, std::ios::end);
  std::streamsize n = in.tellg();
  in.seekg(0);
  std::vector<double> v(n / sizeof(double));
  in.read(reinterpret_cast<char*>(v.data()), n);
  return v;
}

void write_doubles(const std::string& file, const std::vector<double>& v) {
  std::ofstream out(file, std::ios::binary);
  if (!out) die("cannot write " + file);
  out.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(double));
}

// Row-major offset of an Index in an Array of the given dimensions (last index fastest).
long offset(const Index& pos, const Dim_array& dims) {
  long o = 0;
  for (int k = 0; k < dims.get_ndim(); k++) o = o * dims(k) + pos(k);
  return o;
}

struct Problem {
  std::unique_ptr<Space_spheric> space;
  std::unique_ptr<System_of_eqs> syst;
  std::unique_ptr<Base_tensor> basis;
  std::unique_ptr<Metric_flat> metric;
  std::map<std::string, std::unique_ptr<Tensor>> tensors;
  std::vector<std::string> unknowns;  // add_var order
  std::vector<double*> doubles;

  int ndom() const { return space->get_nbr_domains(); }

  // Sets a scalar's collocation values from SRC starting at `at`, returns the next offset.
  size_t fill(Scalar& s, const std::string& src, size_t at) {
    char* end = nullptr;
    double cst = std::strtod(src.c_str(), &end);
    bool is_number = end && *end == '\0';
    std::vector<double> vals;
    if (!is_number) vals = read_doubles(src);
    for (int d = 0; d < ndom(); d++) {
      const Dim_array& np = space->get_domain(d)->get_nbr_points();
      Val_domain& vd = s.set_domain(d);
      vd.allocate_conf();
      Index pos(np);
      long n = 1;
      for (int k = 0; k < np.get_ndim(); k++) n *= np(k);
      do {
        double v = is_number ? cst : vals.at(at + offset(pos, np));
        vd.set(pos) = v;
      } while (pos.inc());
      if (!is_number) at += n;
    }
    return at;
  }

  void set_base(Scalar& s, const std::string& kind) {
    for (int d = 0; d < ndom(); d++) {
      if (kind == "std") s.std_base_domain(d);
      else if (kind == "anti") s.std_anti_base_domain(d);
      else if (kind == "xcart") s.std_base_x_cart_domain(d);
      else if (kind == "ycart") s.std_base_y_cart_domain(d);
      else if (kind == "zcart") s.std_base_z_cart_domain(d);
      else die("unknown base kind " + kind);
    }
  }

  // Sets a scalar's coefficients from FILE (domain by domain); the base must be set first.
  void fill_coefs(Scalar& s, const std::string& file) {
    std::vector<double> vals = read_doubles(file);
    size_t at = 0;
    for (int d = 0; d < ndom(); d++) {
      const Dim_array& nc = space->get_domain(d)->get_nbr_coefs();
      Val_domain& vd = s.set_domain(d);
      vd.allocate_coef();
      Index pos(nc);
      long n = 1;
      for (int k = 0; k < nc.get_ndim(); k++) n *= nc(k);
      do {
        vd.set_coef(pos) = vals.at(at + offset(pos, nc));
      } while (pos.inc());
      at += n;
    }
  }

  // Collocation values of one tensor, component by component, domain by domain.
  std::vector<double> conf_values(const std::string& name) {
    std::vector<double> out;
    Tensor& t = *tensors.at(name);
    for (int c = 0; c < t.get_n_comp(); c++) {
      const Scalar& s = t.get_valence() == 0 ? static_cast<Scalar&>(t) : t.set(c + 1);
      for (int d = 0; d < ndom(); d++) {
        const Dim_array& np = space->get_domain(d)->get_nbr_points();
        long n = 1;
        for (int k = 0; k < np.get_ndim(); k++) n *= np(k);
        const Val_domain& vd = s(d);
        if (vd.check_if_zero()) {
          out.insert(out.end(), n, 0.0);
          continue;
        }
        vd.coef_i();
        Array<double> cv(vd.get_conf());
        out.insert(out.end(), cv.get_data(), cv.get_data() + n);
      }
    }
    return out;
  }

  // Coefficients of one tensor, component by component, domain by domain.
  std::vector<double> coefs(const std::string& name) {
    std::vector<double> out;
    Tensor& t = *tensors.at(name);
    for (int c = 0; c < t.get_n_comp(); c++) {
      const Scalar& s = t.get_valence() == 0 ? static_cast<Scalar&>(t) : t.set(c + 1);
      for (int d = 0; d < ndom(); d++) {
        const Dim_array& nc = space->get_domain(d)->get_nbr_coefs();
        long n = 1;
        for (int k = 0; k < nc.get_ndim(); k++) n *= nc(k);
        const Val_domain& vd = s(d);
        if (vd.check_if_zero()) {
          out.insert(out.end(), n, 0.0);
          continue;
        }
        vd.coef();
        Array<double> cf(vd.get_coef());
        out.insert(out.end(), cf.get_data(), cf.get_data() + n);
      }
    }
    return out;
  }

  // Coefficients of every unknown, component by component, domain by domain.
  std::vector<double> field_coefs() {
    std::vector<double> out;
    for (const auto& name : unknowns) {
      std::vector<double> one = coefs(name);
      out.insert(out.end(), one.begin(), one.end());
    }
    return out;
  }
};

std::vector<double> to_vector(const Array<double>& a) {
  return std::vector<double>(a.get_data(), a.get_data() + a.get_size(0));
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 2) die("usage: ref_newton SPEC");
  std::ifstream spec(argv[1]);
  if (!spec) die(std::string("cannot open ") + argv[1]);
  Problem P;
  std::string line;
  while (std::getline(spec, line)) {
    if (line.empty() || line[0] == '#') continue;
    std::string head = line, text;
    size_t bar = line.find('|');
    std::vector<std::string> strs;
    if (bar != std::string::npos) {
      head = line.substr(0, bar);
      std::string rest = line.substr(bar + 1);
      size_t p;
      while ((p = rest.find('|')) != std::string::npos) {
        strs.push_back(rest.substr(0, p));
        rest = rest.substr(p + 1);
      }
      strs.push_back(rest);
      for (auto& s : strs) {
        size_t a = s.find_first_not_of(' '), b = s.find_last_not_of(' ');
        s = a == std::string::npos ? "" : s.substr(a, b - a + 1);
      }
    }
    std::istringstream ts(head);
    std::string cmd;
    ts >> cmd;
    if (cmd == "space") {
      int nr, nt, np, nb;
      ts >> nr >> nt >> np >> nb;
      Array<double> bounds(nb);
      for (int i = 0; i < nb; i++) ts >> bounds.set(i);
      Dim_array res(3);
      res.set(0) = nr;
      res.set(1) = nt;
      res.set(2) = np;
      Point center(3);
      for (int i = 1; i <= 3; i++) center.set(i) = 0;
      P.space.reset(new Space_spheric(CHEB_TYPE, center, res, bounds));
      P.basis.reset(new Base_tensor(*P.space, CARTESIAN_BASIS));
    } else if (cmd == "system") {
      int a, b;
      ts >> a >> b;
      P.syst.reset(new System_of_eqs(*P.space, a, b));
    } else if (cmd == "metric_flat") {
      std::string name;
      ts >> name;
      P.metric.reset(new Metric_flat(*P.space, *P.basis));
      P.metric->set_system(*P.syst, name.c_str());
    } else if (cmd == "scalar") {
      std::string name, kind, src;
      ts >> name >> kind >> src;
      auto* s = new Scalar(*P.space);
      P.fill(*s, src, 0);
      P.set_base(*s, kind);
      P.tensors[name].reset(s);
    } else if (cmd == "scalar_c") {
      std::string name, kind, file;
      ts >> name >> kind >> file;
      auto* s = new Scalar(*P.space);
      P.set_base(*s, kind);
      P.fill_coefs(*s, file);
      P.tensors[name].reset(s);
    } else if (cmd == "dump_coefs") {
      std::string name, file;
      ts >> name >> file;
      write_doubles(file, P.coefs(name));
    } else if (cmd == "dump_conf") {
      std::string name, file;
      ts >> name >> file;
      write_doubles(file, P.conf_values(name));
    } else if (cmd == "vector") {
      std::string name, src;
      ts >> name >> src;
      auto* v = new Vector(*P.space, CON, *P.basis);
      size_t at = 0;
      for (int c = 1; c <= 3; c++) at = P.fill(v->set(c), src, at);
      v->std_base();
      P.tensors[name].reset(v);
    } else if (cmd == "var") {
      std::string name;
      ts >> name;
      P.syst->add_var(name.c_str(), *P.tensors.at(name));
      P.unknowns.push_back(name);
    } else if (cmd == "cst") {
      std::string name;
      ts >> name;
      P.syst->add_cst(name.c_str(), *P.tensors.at(name));
    } else if (cmd == "cstd") {
      std::string name;
      double v;
      ts >> name >> v;
      P.syst->add_cst(name.c_str(), v);
    } else if (cmd == "def") {
      P.syst->add_def(strs.at(0).c_str());
    } else if (cmd == "defd") {
      int d;
      ts >> d;
      P.syst->add_def(d, strs.at(0).c_str());
    } else if (cmd == "inside") {
      int d;
      ts >> d;
      P.syst->add_eq_inside(d, strs.at(0).c_str());
    } else if (cmd == "bc") {
      int d, b;
      ts >> d >> b;
      P.syst->add_eq_bc(d, b, strs.at(0).c_str());
    } else if (cmd == "matching") {
      int d, b;
      ts >> d >> b;
      P.syst->add_eq_matching(d, b, strs.at(0).c_str());
    } else if (cmd == "full") {
      int d;
      ts >> d;
      P.syst->add_eq_full(d, strs.at(0).c_str());
    } else if (cmd == "firstint") {
      int a, b;
      ts >> a >> b;
      P.syst->add_eq_first_integral(a, b, strs.at(0).c_str(), strs.at(1).c_str());
    } else if (cmd == "dump_residual") {
      std::string file;
      ts >> file;
      P.syst->vars_to_terms();
      write_doubles(file, to_vector(P.syst->sec_member()));
    } else if (cmd == "dump_cols") {
      std::string file;
      ts >> file;
      P.syst->vars_to_terms();
      P.syst->sec_member();
      std::vector<double> out;
      int c;
      while (ts >> c) {
        std::vector<double> col = to_vector(P.syst->do_col_J(c));
        out.insert(out.end(), col.begin(), col.end());
      }
      write_doubles(file, out);
    } else if (cmd == "dump_jx") {
      std::string xfile, file;
      ts >> xfile >> file;
      std::vector<double> x = read_doubles(xfile);
      Array<double> xx(static_cast<int>(x.size()));
      for (size_t i = 0; i < x.size(); i++) xx.set(static_cast<int>(i)) = x[i];
      P.syst->vars_to_terms();
      P.syst->sec_member();
      write_doubles(file, to_vector(P.syst->do_JX(xx)));
    } else if (cmd == "dump_fields") {
      std::string file;
      ts >> file;
      write_doubles(file, P.field_coefs());
    } else if (cmd == "newton") {
      double prec;
      int maxsteps;
      std::string prefix;
      ts >> prec >> maxsteps >> prefix;
      std::vector<double> errors;
      bool done = false;
      for (int k = 0; k < maxsteps && !done; k++) {
        double err = 0;
        done = P.syst->do_newton_seq(prec, err);
        errors.push_back(err);
        if (!done) write_doubles(prefix + "_step" + std::to_string(k) + ".bin", P.field_coefs());
      }
      write_doubles(prefix + "_errors.bin", errors);
      if (!done) die("no convergence");
    } else {
      die("unknown command " + cmd);
    }
  }
  return 0;
}
