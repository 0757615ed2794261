// Built-in PDE operators: the compute_rhs / compute_lhs callbacks of the reference
// applications, written against the device FieldContainer API exactly as an application
// writes them (same getters, setters, dependency types and block ids). Each class is
// trivially copyable and travels to the GPU as a kernel argument.
//
//   AllenCahn        applications/allen_cahn/explicit/custom_pde.h:72-101
//   CahnHilliard     applications/cahn_hilliard/explicit/custom_pde.h:91-131
//   Eshelby          applications/mechanics/eshelby_inclusion/custom_pde.h:55-92, with the
//                    eigenstrain of seeded spherical inclusions used by the 3-D elasticity
//                    workload (a sum of tanh profiles capped at one)
//   CoupledACCH      applications/coupled_allen_cahn_cahn_hilliard/custom_pde.h:63-176
#pragma once

#include <prismspf/core/field_container.h>
#include <prismspf/utilities/mechanics.h>

#ifndef PPF_ESHELBY_F32_MIN_BLOCKS
#define PPF_ESHELBY_F32_MIN_BLOCKS 6
#endif

namespace ppf {

using namespace prismspf;

template <unsigned int dim, unsigned int degree, typename number>
struct AllenCahn {
  using ScalarValue = dealii::VectorizedArray<number>;
  using ScalarGrad = dealii::Tensor<1, dim, ScalarValue>;
  number m_well;
  number kappa;

  PPF_HD void compute_rhs(FieldContainer<dim, degree, number>& variable_list, const SimulationTimer& sim_timer,
                          unsigned int solve_block_id) const {
    if (solve_block_id == 1) {
      ScalarValue n_val = variable_list.template get_value<Scalar, OldOne>(0);
      ScalarGrad n_grad = variable_list.template get_gradient<Scalar, OldOne>(0);
      ScalarValue f_well = 4.0 * n_val * (n_val - 1.0) * (n_val - 0.5);
      ScalarValue eq_n = n_val - sim_timer.get_timestep() * m_well * f_well;
      ScalarGrad eqx_n = -sim_timer.get_timestep() * kappa * m_well * n_grad;
      variable_list.set_value_term(0, eq_n);
      variable_list.set_gradient_term(0, eqx_n);
    } else if (solve_block_id == 2) {
      ScalarValue n_val = variable_list.template get_value<Scalar, Current>(0);
      ScalarGrad n_grad = variable_list.template get_gradient<Scalar, Current>(0);
      ScalarValue f_chem = n_val * n_val * n_val * n_val - 2.0 * n_val * n_val * n_val + n_val * n_val;
      ScalarValue f_grad = 0.5 * kappa * n_grad.norm_square();
      variable_list.set_value_term(1, n_grad.norm());
      variable_list.set_value_term(2, f_chem + f_grad);
    }
  }
  PPF_HD void compute_lhs(FieldContainer<dim, degree, number>&, const SimulationTimer&, unsigned int) const {}
};

template <unsigned int dim, unsigned int degree, typename number>
struct CahnHilliard {
  using ScalarValue = dealii::VectorizedArray<number>;
  using ScalarGrad = dealii::Tensor<1, dim, ScalarValue>;
  // Q2 3-D: 32 registers and 8 resident blocks per SM measured 2.7 % faster than the free
  // register budget (6 blocks), despite a 60-byte spill
  static constexpr int cell_min_blocks = (dim == 3 && degree == 2) ? 8 : 1;
  number McV;
  number KcV;
  number WcV;

  PPF_HD void compute_rhs(FieldContainer<dim, degree, number>& variable_list, const SimulationTimer& sim_timer,
                          unsigned int solve_block_id) const {
    if (solve_block_id == 0) {
      ScalarValue c = variable_list.template get_value<Scalar, OldOne>(0);
      ScalarGrad mux = variable_list.template get_gradient<Scalar, OldOne>(1);
      ScalarValue eq_c = c;
      ScalarGrad eqx_c = -McV * sim_timer.get_timestep() * mux;
      variable_list.set_value_term(0, eq_c);
      variable_list.set_gradient_term(0, eqx_c);
    } else if (solve_block_id == 1) {
      ScalarValue c = variable_list.template get_value<Scalar, Current>(0);
      ScalarGrad cx = variable_list.template get_gradient<Scalar, Current>(0);
      ScalarValue fcV = WcV * c * (c - 1.0) * (c - 0.5);
      ScalarGrad eqx_mu = KcV * cx;
      variable_list.set_value_term(1, fcV);
      variable_list.set_gradient_term(1, eqx_mu);
    } else if (solve_block_id == 2) {
      ScalarValue c = variable_list.template get_value<Scalar, Current>(0);
      ScalarGrad cx = variable_list.template get_gradient<Scalar, Current>(0);
      ScalarValue f_chem = c * c * c * c - 2.0 * c * c * c + c * c;
      ScalarValue f_grad = 0.5 * KcV * cx.norm_square();
      variable_list.set_value_term(2, f_chem + f_grad);
    }
  }
  PPF_HD void compute_lhs(FieldContainer<dim, degree, number>&, const SimulationTimer&, unsigned int) const {}
};

constexpr int ESHELBY_MAX_INCLUSIONS = 64;

template <unsigned int dim, unsigned int degree, typename number>
struct Eshelby {
  using ScalarValue = dealii::VectorizedArray<number>;
  using VectorGrad = dealii::Tensor<2, dim, ScalarValue>;
  // register budget of the FP32 operator (the multigrid smoothing levels)
  static constexpr int cell_min_blocks = std::is_same_v<number, float> ? PPF_ESHELBY_F32_MIN_BLOCKS : 1;
  // the FP64 left-hand side runs on the warp-resident kernel (measured: the 64^3 Q2 GMG-CG
  // iterations 282 ms against 307 ms on the thread-block tiles), 64 registers, no spill
  static constexpr bool cell_warp_lhs = true;
  static constexpr int cell_warp_min_blocks = 4;
  static constexpr unsigned int nv = Mechanics::voigt_tensor_size<dim>;
  dealii::Tensor<2, nv, number> stiffness;
  number e0;      // eigenstrain magnitude
  number width;   // tanh interface width
  int n_incl;     // 0: the application's single inclusion of radius 10 at the origin
  number incl[ESHELBY_MAX_INCLUSIONS][4];  // centre xyz, radius

  PPF_HD ScalarValue strain_magnitude(const dealii::Point<dim, ScalarValue>& p) const {
    if (n_incl == 0) {
      ScalarValue dist_from_inclusion = p.norm();
      ScalarValue inclusion_radius(10.0);
      return 0.01 * (0.5 + 0.5 * std::tanh(10.0 * (dist_from_inclusion - inclusion_radius)));
    }
    // an inclusion farther than its radius + 20 widths adds 0.5 (1 - tanh(x)) < e^-40 (below
    // FP64 resolution of the sum); skipping it on the squared distance saves the sqrt and tanh
    ScalarValue s(0.0);
    for (int i = 0; i < n_incl; ++i) {
      ScalarValue r2(0.0);
      for (unsigned int d = 0; d < dim; ++d) {
        ScalarValue dx = p[d] - incl[i][d];
        r2 += dx * dx;
      }
      const number reach = incl[i][3] + number(20) * width;
      if (r2.v > reach * reach) continue;
      s += 0.5 * (1.0 - std::tanh((std::sqrt(r2) - incl[i][3]) / width));
    }
    return e0 * std::min(s, ScalarValue(1.0));
  }

  PPF_HD void compute_rhs(FieldContainer<dim, degree, number>& variable_list, const SimulationTimer&,
                          unsigned int solve_block_id) const {
    if (solve_block_id == 1) {
      ScalarValue strain_value = strain_magnitude(variable_list.get_q_point_location());
      VectorGrad transformation_strain;
      for (unsigned int i = 0; i < dim; i++) transformation_strain[i][i] = strain_value;
      VectorGrad stress;
      Mechanics::compute_stress<dim, ScalarValue>(stiffness, transformation_strain, stress);
      variable_list.set_gradient_term(0, -stress);
    }
  }

  PPF_HD void compute_lhs(FieldContainer<dim, degree, number>& variable_list, const SimulationTimer&,
                          unsigned int solve_block_id) const {
    if (solve_block_id == 1) {
      VectorGrad ux = variable_list.template get_symmetric_gradient<Vector, LHS>(0);
      VectorGrad stress;
      Mechanics::compute_stress<dim, ScalarValue>(stiffness, ux, stress);
      variable_list.set_gradient_term(0, stress);
    }
  }
};

template <unsigned int dim, unsigned int degree, typename number>
struct CoupledACCH {
  using ScalarValue = dealii::VectorizedArray<number>;
  using ScalarGrad = dealii::Tensor<1, dim, ScalarValue>;
  number Mc;
  number Mn;
  number Kn;

  PPF_HD void compute_rhs(FieldContainer<dim, degree, number>& variable_list, const SimulationTimer& sim_timer,
                          unsigned int solve_block_id) const {
    const double dt = sim_timer.get_timestep();
    constexpr double a0 = -1.6704;
    constexpr double a1 = -4.776;
    constexpr double a2 = 5.1622;
    constexpr double a3 = -2.7375;
    constexpr double a4 = 1.3687;
    constexpr double b0 = -1.5924;
    constexpr double b1 = -5.9746;
    constexpr double b2 = 5.0;
    if (solve_block_id == 0) {
      const ScalarValue c = variable_list.template get_value<Scalar, OldOne>(0);
      const ScalarGrad cx = variable_list.template get_gradient<Scalar, OldOne>(0);
      const ScalarValue n = variable_list.template get_value<Scalar, OldOne>(1);
      const ScalarGrad nx = variable_list.template get_gradient<Scalar, OldOne>(1);
      const ScalarValue c2 = c * c;
      const ScalarValue c3 = c * c2;
      const ScalarValue c4 = c2 * c2;
      const ScalarValue n2 = n * n;
      const ScalarValue n3 = n * n2;
      const ScalarValue n4 = n2 * n2;
      const ScalarValue n5 = n * n4;
      ScalarValue fa = a0 + a1 * c + a2 * c2 + a3 * c3 + a4 * c4;
      ScalarValue fa_c = a1 + 2 * a2 * c + 3 * a3 * c2 + 4 * a4 * c3;
      ScalarValue fa_cc = 2 * a2 + 6 * a3 * c + 12 * a4 * c2;
      ScalarValue fb = b0 + b1 * c + b2 * c2;
      ScalarValue fb_c = b1 + 2 * b2 * c;
      ScalarValue fb_cc = ScalarValue(2 * b2);
      ScalarValue h = 10.0 * n3 - 15.0 * n4 + 6.0 * n5;
      ScalarValue hn = 30.0 * n2 - 60.0 * n3 + 30.0 * n4;
      ScalarGrad mu_grad = -(cx * ((1.0 - h) * fa_cc + h * fb_cc) + nx * ((fb_c - fa_c) * hn));
      ScalarGrad dcdt_vec = ScalarValue(Mc) * -mu_grad;
      ScalarValue dndt_val = -Mn * (fb - fa) * hn;
      ScalarGrad dndt_vec = ScalarValue(Kn * Mn) * nx;
      variable_list.set_value_term(0, c);
      variable_list.set_gradient_term(0, -dt * dcdt_vec);
      variable_list.set_value_term(1, n + dt * dndt_val);
      variable_list.set_gradient_term(1, -dt * dndt_vec);
    } else if (solve_block_id == 1) {
      const ScalarValue c = variable_list.template get_value<Scalar, Current>(0);
      const ScalarGrad cx = variable_list.template get_gradient<Scalar, Current>(0);
      const ScalarValue n = variable_list.template get_value<Scalar, Current>(1);
      const ScalarGrad nx = variable_list.template get_gradient<Scalar, Current>(1);
      const ScalarValue c2 = c * c;
      const ScalarValue c3 = c * c2;
      const ScalarValue c4 = c2 * c2;
      const ScalarValue n2 = n * n;
      const ScalarValue n3 = n * n2;
      const ScalarValue n4 = n2 * n2;
      const ScalarValue n5 = n * n4;
      ScalarValue fa = a0 + a1 * c + a2 * c2 + a3 * c3 + a4 * c4;
      ScalarValue fb = b0 + b1 * c + b2 * c2;
      ScalarValue h = 10.0 * n3 - 15.0 * n4 + 6.0 * n5;
      ScalarValue f_chem = (1.0 - h) * fa + h * fb;
      ScalarValue f_grad = 0.5 * Kn * nx * nx;
      variable_list.set_value_term(2, f_chem + f_grad);
      variable_list.set_value_term(3, cx.norm());
    }
  }
  PPF_HD void compute_lhs(FieldContainer<dim, degree, number>&, const SimulationTimer&, unsigned int) const {}
};

// ------------------------------------------------------------------------------------------
// Hand-written linearisations of the coupled model's explicit block (block 0 above).
//
// Per quadrature point the block maps the inputs x = (c, grad c, n, grad n) to the submitted
// terms y = (v_c, g_c, v_n, g_n):
//   A = (1-h) fa'' + h fb'',  B = (fb' - fa') h'
//   v_c = c,  g_c = -dt Mc (A grad c + B grad n)
//   v_n = n - dt Mn (fb - fa) h',  g_n = -dt Kn Mn grad n
// The explicit step is u+ = invM (.) R(u) with R the integrated terms. Its Jacobian is applied
// pointwise through dy/dx:
//   CoupledACCHTangent: dy = (dy/dx) dx + (dy/dtheta) dtheta, integrated like the forward terms
//                       (tangent-linear step, dtheta = (dMc, dKn) from the constants);
//   CoupledACCHAdjoint: given w = invM (.) lambda evaluated as (W, grad W) per field, submits
//                       (dy/dx)^T w as value/gradient terms (the transposed sum-factorised
//                       apply gives (dR/du)^T w) and w.(dy/dMc), w.(dy/dKn) as value terms of
//                       two extra fields whose nodal sums are the parameter gradients.
// Field indices inside these operators: inputs u = (c, n) as fields 0, 1 at age Current, the
// direction (dx or w) as fields 0, 1 at age SRC; outputs fields 0, 1 (and 2, 3 for dMc, dKn).
// ------------------------------------------------------------------------------------------
template <typename number>
struct ACCHPoint {
  number A, B, A_c, A_n, B_c, B_n, dvn_dc, dvn_dn, gc_dMc_fac;
  number fbfa_hn;  // (fb - fa) h'
};

template <typename number>
PPF_HD ACCHPoint<number> acch_point(number c, number n) {
  constexpr double a1 = -4.776, a2 = 5.1622, a3 = -2.7375, a4 = 1.3687;
  constexpr double a0 = -1.6704, b0 = -1.5924, b1 = -5.9746, b2 = 5.0;
  const number c2 = c * c, c3 = c2 * c, c4 = c2 * c2;
  const number n2 = n * n, n3 = n2 * n, n4 = n2 * n2, n5 = n4 * n;
  const number fa = a0 + a1 * c + a2 * c2 + a3 * c3 + a4 * c4;
  const number fa_c = a1 + 2 * a2 * c + 3 * a3 * c2 + 4 * a4 * c3;
  const number fa_cc = 2 * a2 + 6 * a3 * c + 12 * a4 * c2;
  const number fa_ccc = 6 * a3 + 24 * a4 * c;
  const number fb = b0 + b1 * c + b2 * c2;
  const number fb_c = b1 + 2 * b2 * c;
  const number fb_cc = 2 * b2;
  const number h = 10.0 * n3 - 15.0 * n4 + 6.0 * n5;
  const number hn = 30.0 * n2 - 60.0 * n3 + 30.0 * n4;
  const number hnn = 60.0 * n - 180.0 * n2 + 120.0 * n3;
  ACCHPoint<number> p;
  p.A = (1.0 - h) * fa_cc + h * fb_cc;
  p.B = (fb_c - fa_c) * hn;
  p.A_c = (1.0 - h) * fa_ccc;
  p.A_n = hn * (fb_cc - fa_cc);
  p.B_c = (fb_cc - fa_cc) * hn;
  p.B_n = (fb_c - fa_c) * hnn;
  p.dvn_dc = (fb_c - fa_c) * hn;  // times -dt Mn
  p.dvn_dn = (fb - fa) * hnn;     // times -dt Mn
  p.fbfa_hn = (fb - fa) * hn;
  p.gc_dMc_fac = 0.0;
  return p;
}

template <unsigned int dim, unsigned int degree, typename number>
struct CoupledACCHTangent {
  using ScalarValue = dealii::VectorizedArray<number>;
  using ScalarGrad = dealii::Tensor<1, dim, ScalarValue>;
  number Mc, Mn, Kn;
  number dMc, dKn;  // parameter direction

  PPF_HD void compute_rhs(FieldContainer<dim, degree, number>& vl, const SimulationTimer& t, unsigned int) const {
    const number dt = t.get_timestep();
    const number c = vl.template get_value<Scalar, Current>(0).v;
    const number n = vl.template get_value<Scalar, Current>(1).v;
    const ScalarGrad cx = vl.template get_gradient<Scalar, Current>(0);
    const ScalarGrad nx = vl.template get_gradient<Scalar, Current>(1);
    const number dc = vl.template get_value<Scalar, SRC>(0).v;
    const number dn = vl.template get_value<Scalar, SRC>(1).v;
    const ScalarGrad dcx = vl.template get_gradient<Scalar, SRC>(0);
    const ScalarGrad dnx = vl.template get_gradient<Scalar, SRC>(1);
    const ACCHPoint<number> p = acch_point<number>(c, n);
    ScalarGrad gc, gn;
    for (unsigned int d = 0; d < dim; ++d) {
      const number lin = (p.A_c * cx[d].v + p.B_c * nx[d].v) * dc + (p.A_n * cx[d].v + p.B_n * nx[d].v) * dn +
                         p.A * dcx[d].v + p.B * dnx[d].v;
      gc[d] = -dt * Mc * lin - dt * dMc * (p.A * cx[d].v + p.B * nx[d].v);
      gn[d] = -dt * Kn * Mn * dnx[d].v - dt * dKn * Mn * nx[d].v;
    }
    vl.set_value_term(0, ScalarValue(dc));
    vl.set_gradient_term(0, gc);
    vl.set_value_term(1, ScalarValue(dn - dt * Mn * (p.dvn_dc * dc + p.dvn_dn * dn)));
    vl.set_gradient_term(1, gn);
  }
  PPF_HD void compute_lhs(FieldContainer<dim, degree, number>&, const SimulationTimer&, unsigned int) const {}
};

template <unsigned int dim, unsigned int degree, typename number>
struct CoupledACCHAdjoint {
  using ScalarValue = dealii::VectorizedArray<number>;
  using ScalarGrad = dealii::Tensor<1, dim, ScalarValue>;
  number Mc, Mn, Kn;

  PPF_HD void compute_rhs(FieldContainer<dim, degree, number>& vl, const SimulationTimer& t, unsigned int) const {
    const number dt = t.get_timestep();
    const number c = vl.template get_value<Scalar, Current>(0).v;
    const number n = vl.template get_value<Scalar, Current>(1).v;
    const ScalarGrad cx = vl.template get_gradient<Scalar, Current>(0);
    const ScalarGrad nx = vl.template get_gradient<Scalar, Current>(1);
    const number Wc = vl.template get_value<Scalar, SRC>(0).v;
    const number Wn = vl.template get_value<Scalar, SRC>(1).v;
    const ScalarGrad Wcx = vl.template get_gradient<Scalar, SRC>(0);
    const ScalarGrad Wnx = vl.template get_gradient<Scalar, SRC>(1);
    const ACCHPoint<number> p = acch_point<number>(c, n);
    // (dy/dx)^T w
    number ac = Wc - dt * Mn * p.dvn_dc * Wn;  // value entries
    number an = Wn - dt * Mn * p.dvn_dn * Wn;
    ScalarGrad gc, gn;
    number dMc = 0.0, dKn = 0.0;
    for (unsigned int d = 0; d < dim; ++d) {
      const number wgc = Wcx[d].v, wgn = Wnx[d].v;
      ac += -dt * Mc * (p.A_c * cx[d].v + p.B_c * nx[d].v) * wgc;
      an += -dt * Mc * (p.A_n * cx[d].v + p.B_n * nx[d].v) * wgc;
      gc[d] = -dt * Mc * p.A * wgc;
      gn[d] = -dt * Mc * p.B * wgc - dt * Kn * Mn * wgn;
      dMc += -dt * (p.A * cx[d].v + p.B * nx[d].v) * wgc;
      dKn += -dt * Mn * nx[d].v * wgn;
    }
    vl.set_value_term(0, ScalarValue(ac));
    vl.set_gradient_term(0, gc);
    vl.set_value_term(1, ScalarValue(an));
    vl.set_gradient_term(1, gn);
    vl.set_value_term(2, ScalarValue(dMc));
    vl.set_value_term(3, ScalarValue(dKn));
  }
  PPF_HD void compute_lhs(FieldContainer<dim, degree, number>&, const SimulationTimer&, unsigned int) const {}
};

}  // namespace ppf

namespace ppf {

// applications/allen_cahn/implicit/custom_pde.h:70-125: backward Euler through a Newton block
// (block 1: residual old_n - n - dt M f'(n), Jacobian (1 + dt M f''(n)) dn + dt kappa M grad dn)
// and the post-processing block 2 of the explicit application.
template <unsigned int dim, unsigned int degree, typename number>
struct AllenCahnImplicit {
  using ScalarValue = dealii::VectorizedArray<number>;
  using ScalarGrad = dealii::Tensor<1, dim, ScalarValue>;
  number m_well;
  number kappa;

  PPF_HD void compute_rhs(FieldContainer<dim, degree, number>& variable_list, const SimulationTimer& sim_timer,
                          unsigned int solve_block_id) const {
    if (solve_block_id == 1) {
      ScalarValue n = variable_list.template get_value<Scalar, Current>(0);
      ScalarGrad nx = variable_list.template get_gradient<Scalar, Current>(0);
      ScalarValue old_n = variable_list.template get_value<Scalar, OldOne>(0);
      ScalarValue f_well = 4.0 * n * (n - 1.0) * (n - 0.5);
      const number dt = number(sim_timer.get_timestep());
      variable_list.set_value_term(0, old_n - n - dt * m_well * f_well);
      variable_list.set_gradient_term(0, -dt * kappa * m_well * nx);
    } else if (solve_block_id == 2) {
      ScalarValue n = variable_list.template get_value<Scalar, Current>(0);
      ScalarGrad nx = variable_list.template get_gradient<Scalar, Current>(0);
      ScalarValue f_chem = n * n * n * n - 2.0 * n * n * n + n * n;
      variable_list.set_value_term(1, nx.norm());
      variable_list.set_value_term(2, f_chem + 0.5 * kappa * nx.norm_square());
    }
  }

  PPF_HD void compute_lhs(FieldContainer<dim, degree, number>& variable_list, const SimulationTimer& sim_timer,
                          unsigned int solve_block_id) const {
    if (solve_block_id == 1) {
      ScalarValue n = variable_list.template get_value<Scalar, Current>(0);
      ScalarValue dn = variable_list.template get_value<Scalar, Change>(0);
      ScalarGrad dnx = variable_list.template get_gradient<Scalar, Change>(0);
      ScalarValue df_well = 12.0 * n * (n - 1.0) + 2.0;
      const number dt = number(sim_timer.get_timestep());
      variable_list.set_value_term(0, dn * (1.0 + dt * m_well * df_well));
      variable_list.set_gradient_term(0, dt * kappa * m_well * dnx);
    }
  }
};

// applications/cahn_hilliard/implicit/custom_pde.h:90-160: one Newton block over (c, mu)
// (block 0) and the post-processing block 2.
template <unsigned int dim, unsigned int degree, typename number>
struct CahnHilliardImplicit {
  using ScalarValue = dealii::VectorizedArray<number>;
  using ScalarGrad = dealii::Tensor<1, dim, ScalarValue>;
  number McV;
  number KcV;
  number WcV;

  PPF_HD void compute_rhs(FieldContainer<dim, degree, number>& variable_list, const SimulationTimer& sim_timer,
                          unsigned int solve_block_id) const {
    const number dt = number(sim_timer.get_timestep());
    if (solve_block_id == 0) {
      ScalarValue c = variable_list.template get_value<Scalar, Current>(0);
      ScalarGrad cx = variable_list.template get_gradient<Scalar, Current>(0);
      ScalarValue mu = variable_list.template get_value<Scalar, Current>(1);
      ScalarGrad mux = variable_list.template get_gradient<Scalar, Current>(1);
      ScalarValue c_old = variable_list.template get_value<Scalar, OldOne>(0);
      variable_list.set_value_term(0, c_old - c);
      variable_list.set_gradient_term(0, -(dt * McV * mux));
      variable_list.set_value_term(1, mu - WcV * c * (c - 1.0) * (c - 0.5));
      variable_list.set_gradient_term(1, -(KcV * cx));
    } else if (solve_block_id == 2) {
      ScalarValue c = variable_list.template get_value<Scalar, Current>(0);
      ScalarGrad cx = variable_list.template get_gradient<Scalar, Current>(0);
      ScalarValue f_chem = c * c * c * c - 2.0 * c * c * c + c * c;
      variable_list.set_value_term(2, f_chem + 0.5 * KcV * cx.norm_square());
    }
  }

  PPF_HD void compute_lhs(FieldContainer<dim, degree, number>& variable_list, const SimulationTimer& sim_timer,
                          unsigned int solve_block_id) const {
    const number dt = number(sim_timer.get_timestep());
    if (solve_block_id == 0) {
      ScalarValue c = variable_list.template get_value<Scalar, Current>(0);
      ScalarValue dc = variable_list.template get_value<Scalar, Change>(0);
      ScalarGrad dcx = variable_list.template get_gradient<Scalar, Change>(0);
      ScalarValue dmu = variable_list.template get_value<Scalar, Change>(1);
      ScalarGrad dmux = variable_list.template get_gradient<Scalar, Change>(1);
      ScalarValue j_mu_c = -WcV * (0.5 + 3.0 * (c * (c - 1.0))) * dc;
      variable_list.set_value_term(0, dc);
      variable_list.set_gradient_term(0, dt * McV * dmux);
      variable_list.set_value_term(1, -j_mu_c - dmu);
      variable_list.set_gradient_term(1, KcV * dcx);
    }
  }
};

}  // namespace ppf
