// "Model constant" entries of the parameter file (reference:
// include/prismspf/user_inputs/user_constants.h:33-1000).
//
//   set Model constant <name> = <value>, DOUBLE | INT | BOOL | STRING
//   set Model constant <name> = (x, y, z), TENSOR                 rank 1 (3 values, first dim used)
//   set Model constant <name> = ((a,b,c),(d,e,f),(g,h,i)), TENSOR rank 2 (3x3, leading dim x dim used)
//   set Model constant <name> = (c0, c1, ...), <symmetry> elastic constants [planestress|planestrain]
//
// Elastic constants become the Voigt stiffness matrix (size 2*dim - 1 + dim/3): isotropic
// (E, nu), orthotropic (3-D: E1 E2 E3 nu12 nu13 nu23 G12 G13 G23; 2-D plane stress: E1 E2
// nu12 G12; 2-D plane strain: E1 E2 E3 nu12 nu13 nu23 G12) or anisotropic (3-D: the 21
// entries C11 C22 C33 C44 C55 C66 C12 C13 C14 C15 C16 C23 C24 C25 C26 C34 C35 C36 C45 C46
// C56 in Voigt order xx yy zz yz xz xy; 2-D: C11 C22 C33 C12 C13 C23 over xx yy xy, or the
// 21-entry list reduced to those). 2-D defaults to plane strain.
#pragma once

#include <map>
#include <stdexcept>
#include <string>
#include <variant>
#include <vector>

#include <prismspf/config.h>
#include <prismspf/core/type_enums.h>
#include <prismspf/dealii_shim.h>
#include <prismspf/user_inputs/parameter_file.h>

PRISMS_PF_BEGIN_NAMESPACE

enum StressState { PlaneStress, PlaneStrain, ThreeDimension };

template <unsigned int dim>
class UserConstants {
 public:
  static constexpr int voigt = (2 * dim) - 1 + (dim / 3);
  using Voigt = dealii::Tensor<2, voigt, double>;
  // the Voigt matrix is wrapped so it stays a distinct alternative when voigt == dim (1-D)
  struct Elasticity {
    Voigt C;
  };
  using InputVariant = std::variant<double, int, bool, std::string, dealii::Tensor<1, dim, double>,
                                    dealii::Tensor<2, dim, double>, Elasticity>;

  void add_user_constant(const std::string& name, const std::string& value) {
    model_constants[name] = construct(prm::split_list(value));
  }

  double get_double(const std::string& name) const { return get<double>(name, "double"); }
  int get_int(const std::string& name) const { return get<int>(name, "int"); }
  bool get_bool(const std::string& name) const { return get<bool>(name, "bool"); }
  std::string get_string(const std::string& name) const { return get<std::string>(name, "string"); }
  dealii::Tensor<1, dim> get_rank_1_tensor(const std::string& name) const {
    return get<dealii::Tensor<1, dim, double>>(name, "rank-1 tensor");
  }
  dealii::Tensor<2, dim> get_rank_2_tensor(const std::string& name) const {
    return get<dealii::Tensor<2, dim, double>>(name, "rank-2 tensor");
  }
  Voigt get_elasticity_tensor(const std::string& name) const { return get<Elasticity>(name, "elasticity tensor").C; }

  std::map<std::string, InputVariant> model_constants;

 private:
  template <class T>
  const T& get(const std::string& name, const char* what) const {
    auto it = model_constants.find(name);
    if (it == model_constants.end()) throw std::out_of_range("Model constant '" + name + "' is not defined");
    const T* v = std::get_if<T>(&it->second);
    if (!v) throw std::invalid_argument("Model constant '" + name + "' is not a " + what);
    return *v;
  }

  static bool iequals(const std::string& a, const char* b) {
    const std::string B(b);
    if (a.size() != B.size()) return false;
    for (size_t i = 0; i < a.size(); ++i)
      if (std::tolower(static_cast<unsigned char>(a[i])) != std::tolower(static_cast<unsigned char>(B[i]))) return false;
    return true;
  }

  static std::vector<double> numbers(std::vector<std::string> items) {
    std::vector<double> out;
    for (auto& s : items) {
      std::string t;
      for (char ch : s)
        if (ch != '(' && ch != ')') t += ch;
      out.push_back(prm::to_double(t));
    }
    return out;
  }

  InputVariant construct(std::vector<std::string> parts) {
    if (parts.size() < 2)
      throw std::invalid_argument("At least two fields are required for user-defined variables (value and type).");
    const std::vector<std::string> type = prm::split_list(prm::collapse_blanks(parts.back()), ' ');
    parts.pop_back();
    if (parts.size() == 1) {
      const std::string& v = parts[0];
      if (iequals(type.at(0), "double")) return prm::to_double(v);
      if (iequals(type.at(0), "int")) return prm::to_int(v);
      if (iequals(type.at(0), "bool")) return iequals(v, "true");
      if (iequals(type.at(0), "string")) return v;
      throw std::invalid_argument(
          "The type for user-defined variables must be `double`, `int`, `bool`, `string`, `tensor`, or `elastic "
          "constants`.");
    }
    if (iequals(type.at(0), "tensor")) {
      unsigned int open = 0, close = 0;
      for (auto& s : parts)
        for (char ch : s) open += ch == '(', close += ch == ')';
      if (open != close) throw std::invalid_argument("unbalanced parentheses in a tensor constant");
      const std::vector<double> v = numbers(parts);
      if (open == 1) {
        if (v.size() != 3)
          throw std::invalid_argument("The columns in user-defined constant tensors must be equal to the maximum "
                                      "number of dimensions.");
        dealii::Tensor<1, dim, double> t;
        for (unsigned int i = 0; i < dim; ++i) t[i] = v[i];
        return t;
      }
      if (v.size() != 9) throw std::invalid_argument("matrix constants must be 3x3");
      dealii::Tensor<2, dim, double> t;
      for (unsigned int i = 0; i < dim; ++i)
        for (unsigned int j = 0; j < dim; ++j) t[i][j] = v[3 * i + j];
      return t;
    }
    if (type.size() >= 3 && iequals(type[1], "elastic") && iequals(type[2], "constants")) {
      StressState state = ThreeDimension;
      if (dim == 2) {
        state = PlaneStrain;
        if (type.size() == 4) {
          if (iequals(type[3], "planestress")) state = PlaneStress;
          else if (!iequals(type[3], "planestrain"))
            throw std::invalid_argument("Wrong 2D stress state. Use planestress or planestrain.");
        } else if (type.size() != 3) {
          throw std::invalid_argument("Wrong format of user-defined elastic constants.");
        }
      }
      return Elasticity{stiffness(type[0], numbers(parts), state)};
    }
    throw std::invalid_argument("Only user-defined constant tensors may have multiple elements.");
  }

  static Voigt stiffness(const std::string& symmetry, std::vector<double> c, StressState state) {
    Voigt C;
    auto sym = [&](int i, int j, double v) { C[i][j] = v; C[j][i] = v; };
    if (symmetry == "isotropic") {
      const double E = c.at(0), nu = c.at(1);
      const double mu = E / (2.0 * (1.0 + nu));
      const double lambda = (dim == 2 && state == PlaneStress) ? nu * E / (1.0 - nu * nu)
                                                                : nu * E / ((1.0 + nu) * (1.0 - 2.0 * nu));
      for (int i = 0; i < (int)dim; ++i) {
        for (int j = 0; j < (int)dim; ++j) C[i][j] = lambda;
        C[i][i] = lambda + 2.0 * mu;
      }
      for (int i = dim; i < voigt; ++i) C[i][i] = mu;
      return C;
    }
    if (symmetry == "anisotropic") {
      if (dim == 3) {
        if (c.size() != 21) throw std::invalid_argument("anisotropic elastic constants need 21 entries in 3-D");
        for (int i = 0; i < 6; ++i) C[i][i] = c[i];
        int m = 6;
        for (int i = 0; i < 6; ++i)
          for (int j = i + 1; j < 6; ++j) sym(i, j, c[m++]);
        return C;
      }
      if (c.size() == 21) c = {c[0], c[1], c[5], c[6], c[10], c[14]};
      if (c.size() != 6) throw std::invalid_argument("anisotropic elastic constants need 6 or 21 entries in 2-D");
      C[0][0] = c[0];
      C[1][1] = c[1];
      C[2][2] = c[2];
      sym(0, 1, c[3]);
      sym(0, 2, c[4]);
      sym(1, 2, c[5]);
      return C;
    }
    if (symmetry == "orthotropic") {
      if (dim == 2 && state == PlaneStress) {
        const double E1 = c.at(0), E2 = c.at(1), nu12 = c.at(2), G12 = c.at(3);
        const double nu21 = nu12 * E2 / E1, den = 1.0 - nu12 * nu21;
        C[0][0] = E1 / den;
        C[1][1] = E2 / den;
        sym(0, 1, nu12 * E2 / den);
        C[2][2] = G12;
        return C;
      }
      const double E1 = c.at(0), E2 = c.at(1), E3 = c.at(2), nu12 = c.at(3), nu13 = c.at(4), nu23 = c.at(5);
      const double nu21 = nu12 * E2 / E1, nu31 = nu13 * E3 / E1, nu32 = nu23 * E3 / E2;
      const double delta = 1.0 - nu12 * nu21 - nu23 * nu32 - nu13 * nu31 - 2.0 * nu12 * nu23 * nu31;
      C[0][0] = E1 * (1.0 - nu23 * nu32) / delta;
      C[1][1] = E2 * (1.0 - nu13 * nu31) / delta;
      sym(0, 1, E1 * (nu21 + nu31 * nu23) / delta);
      if (dim == 2) {
        C[2][2] = c.at(6);
        return C;
      }
      C[2][2] = E3 * (1.0 - nu12 * nu21) / delta;
      sym(0, 2, E1 * (nu31 + nu21 * nu32) / delta);
      sym(1, 2, E2 * (nu32 + nu12 * nu31) / delta);
      C[3][3] = c.at(8);
      C[4][4] = c.at(7);
      C[5][5] = c.at(6);
      return C;
    }
    if (symmetry == "transverse")
      throw std::invalid_argument("Transverse elastic tensors haven't been implemented for model constants");
    throw std::invalid_argument("Invalid elasticity tensor type " + symmetry);
  }
};

PRISMS_PF_END_NAMESPACE
