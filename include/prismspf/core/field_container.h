// Device-side FieldContainer: the variable container through which a user callback reads
// dependency values/gradients/hessians and submits value and gradient terms at one
// quadrature point. Same member names, template parameters and meaning as the reference
// (include/prismspf/core/field_container.h:44-586, getters :1065-1256, setters :1258-1314).
//
// GB300 design: one CUDA thread owns one (cell, quadrature point). With Gauss-Lobatto
// collocation the quadrature points are the cell nodes, so values are the gathered nodal
// values and gradients are one 1-D derivative contraction per direction over the node line
// through the point. Nodal values live in shared memory (written by the cell kernel's
// gather); getters contract them on demand, so only what a callback actually asks for is
// computed. Submitted terms are stored pre-multiplied by the integration weights
// (JxW for values, JxW/h_d for gradient component d) for the kernel's integrate step.
#pragma once

#include <prismspf/config.h>
#include <prismspf/core/simulation_timer.h>
#include <prismspf/core/type_enums.h>
#include <prismspf/dealii_shim.h>
#include <prismspf/gpu/fixed_point.cuh>

#include <type_traits>

PRISMS_PF_BEGIN_NAMESPACE

namespace gpu {

constexpr int MAX_FIELDS = 8;
constexpr int NAGE = 6;  // current, old_1..old_4, src
constexpr int MAX_SLOTS = 8;
constexpr int MAX_OUTS = 4;
constexpr int MAX_N = 5;  // up to degree 4
constexpr int LANE_ROW_SLOTS = 8;  // value rows the lane kernel's slot tables cover

enum ErrorBits : int {
  ERR_UNDECLARED_DEPENDENCY = 1,
  ERR_UNDECLARED_SUBMISSION = 2,
  ERR_NONFINITE = 4,
};

PPF_HD constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

PPF_HD constexpr int age_of(DependencyType t) { return t == SRC ? 5 : (t >= Current ? int(t) : -1); }

// Per-launch tables staged in shared memory by the cell kernel (sized for one dim/degree,
// stored in the arithmetic type of the kernel).
template <int dim, int degree, typename number = double>
struct CellTables {
  static constexpr int n = degree + 1;
  static constexpr int nq = ipow(n, dim);
  number Dh[dim][n][n];   // D[q][j] / h_d: derivative of basis j at GL node q, direction d
  number D2h[dim][n][n];  // (D D)[q][j] / h_d^2
  number Dt[n][n];        // Dt[i][j] = D[j][i] (integration uses the transposed derivative)
  number jxw[nq];         // JxW per quadrature point
  // jdt[d][q][j] = D[j][q_d] JxW(q_j) / h_d: the weight, in node q's integral, of the gradient
  // component d submitted (unscaled) at the j-th point q_j of q's line along d
  number jdt[dim][nq][n];
  number lo[3], h[3], gl_x[n];
  number vol;
  signed char slot_of[MAX_FIELDS][NAGE];  // dependency slot of (field, age), -1 if undeclared
  signed char slot_comp0[MAX_SLOTS];      // first value row of a slot
  signed char out_of[MAX_FIELDS];         // output index of a block field, -1 if not in block
  signed char out_row0[MAX_OUTS];         // first output row (per comp: value, then dim grads)
  // integer contractions (FP64 Q1/Q2, prismspf/gpu/fixed_point.cuh); fx = 1 when they apply
  int fx;
  int fx_cubic;                   // the integration scales c_d agree in every direction
  unsigned int fx_rows;           // value rows with a fixed-point copy (those read as gradients)
  signed char wo_sh[dim][nq];     // log2 of the product of w_int(q_e) over the directions e != d,
                                  // w_int = 2w (Q1) or 6w (Q2)
  unsigned long long dsig[3];     // 1/h_d = dsig / 2^63 * 2^dk
  int dk[3];
  unsigned long long isig[3];     // c_d = detJ / (h_d W^dim), W = 2 (Q1) or 6 (Q2): isig / 2^63 * 2^ik
  int ik[3];
  // the lane kernel (prismspf/gpu/cell_kernel_lanes.cuh, cubic cells): value terms are integrated
  // in fixed point as h v next to the gradient terms, with the weight 2^vw_sh[q] = prod_e w_int(q_e)
  // and h = hsig / 2^63 * 2^hk (hpow2: h is a power of two); dpow2[d]: 1/h_d is a power of two
  int fx_lanes;
  int hpow2;
  int hk;
  int dpow2[3];
  unsigned long long hsig;
  signed char vw_sh[nq];
  // the lane kernel keeps a double copy only of the value rows read as values or Hessians
  // (val_rows) and a fixed-point copy only of those read as gradients (fx_rows): slot of row r
  // in each, -1 without one (rows below LANE_ROW_SLOTS)
  unsigned int val_rows;
  signed char lane_vslot[LANE_ROW_SLOTS];
  signed char lane_gslot[LANE_ROW_SLOTS];
};

template <int dim, int degree, typename number = double>
struct CellCtx {
  static constexpr int n = degree + 1;
  static constexpr int nq = ipow(n, dim);
  const CellTables<dim, degree, number>* tab;
  const number* vals;  // [row][stride]
  number* outs;        // [row][stride]
  int stride;          // cells_per_block * nq
  int lc;              // cell within the thread block
  int q;               // quadrature point (= node) within the cell
  int cell[3];         // global cell coordinates
  int* err;
  int submitted;       // bit 2*o: value of output o submitted, bit 2*o+1: gradient
  // integer contractions: fixed-point nodal values [row][stride] and their per-cell block
  // exponents [row][cells per block]; null when the kernel contracts in the arithmetic type
  const long long* vals_fx = nullptr;
  const int* ex_in = nullptr;
  int cpb = 0;
  // Row layout: point q of the thread's cell sits at lc * nq + q, or at q * cpt + lc when cpt > 0
  // (the lane kernel, prismspf/gpu/cell_kernel_lanes.cuh). lean: the lane kernel's all-integer
  // contractions (value terms stored unweighted, derivatives rounded by to_double_fast), with the
  // point's index along each direction in qi.
  int cpt = 0;
  int lean = 0;
  int qi[3] = {0, 0, 0};
  // value terms stored unweighted (a kernel integrating them in fixed point), on any layout
  int raw_values = 0;
};

}  // namespace gpu

template <unsigned int dim, unsigned int degree, typename number>
class FieldContainer {
 public:
  using ScalarValue = dealii::VectorizedArray<number>;
  using VectorValue = dealii::Tensor<1, dim, ScalarValue>;

  template <TensorRank Rank>
  using Value = std::conditional_t<Rank == TensorRank::Scalar || dim == 1, ScalarValue,
                                   dealii::Tensor<int(Rank), dim, ScalarValue>>;
  template <TensorRank Rank>
  using Gradient = dealii::Tensor<int(Rank) + 1, dim, ScalarValue>;
  template <TensorRank Rank>
  using Hessian = dealii::Tensor<int(Rank) + 2, dim, ScalarValue>;

  static constexpr int n = degree + 1;
  static constexpr unsigned int dofs_per_component = gpu::ipow(n, dim);

  using Ctx = gpu::CellCtx<dim, degree, number>;

  PPF_HD explicit FieldContainer(Ctx& c) : ctx(c) {}

  PPF_HD unsigned int get_n_q_points() const { return dofs_per_component; }

  // --- values -------------------------------------------------------------------------
  template <TensorRank Rank, DependencyType type>
  PPF_HD Value<Rank> get_value(unsigned int field_index) const { return get_value<Rank>(field_index, type); }

  template <TensorRank Rank>
  PPF_HD Value<Rank> get_value(unsigned int field_index, DependencyType type) const {
    const int row = row_of(field_index, type);
    if constexpr (Rank == TensorRank::Scalar || dim == 1) {
      return ScalarValue(row < 0 ? number(0) : nodal(row, ctx.q));
    } else {
      Value<Rank> v;
      if (row >= 0)
        for (int c = 0; c < int(dim); ++c) v[c] = nodal(row + c, ctx.q);
      return v;
    }
  }

  // --- gradients ----------------------------------------------------------------------
  template <TensorRank Rank, DependencyType type>
  PPF_HD Gradient<Rank> get_gradient(unsigned int field_index) const { return get_gradient<Rank>(field_index, type); }

  template <TensorRank Rank>
  PPF_HD Gradient<Rank> get_gradient(unsigned int field_index, DependencyType type) const {
    const int row = row_of(field_index, type);
    Gradient<Rank> g;
    if (row < 0) return g;
    if constexpr (Rank == TensorRank::Scalar) {
      for (int d = 0; d < int(dim); ++d) g[d] = deriv(row, d);
    } else {
      for (int c = 0; c < int(dim); ++c)
        for (int d = 0; d < int(dim); ++d) g[c][d] = deriv(row + c, d);
    }
    return g;
  }

  template <TensorRank Rank, DependencyType type>
  PPF_HD dealii::SymmetricTensor<2, dim, ScalarValue> get_symmetric_gradient(unsigned int field_index) const {
    static_assert(Rank == TensorRank::Vector, "Symmetric gradients are only available for vector fields");
    return get_symmetric_gradient<Rank>(field_index, type);
  }

  template <TensorRank Rank>
  PPF_HD dealii::SymmetricTensor<2, dim, ScalarValue> get_symmetric_gradient(unsigned int field_index,
                                                                             DependencyType type) const {
    const Gradient<Rank> g = get_gradient<Rank>(field_index, type);
    dealii::SymmetricTensor<2, dim, ScalarValue> s;
    for (int i = 0; i < int(dim); ++i) {
      s.a[i][i] = g[i][i];
      for (int j = i + 1; j < int(dim); ++j) {
        ScalarValue v = number(0.5) * (g[i][j] + g[j][i]);
        s.a[i][j] = v;
        s.a[j][i] = v;
      }
    }
    return s;
  }

  template <TensorRank Rank, DependencyType type>
  PPF_HD ScalarValue get_divergence(unsigned int field_index) const {
    static_assert(Rank == TensorRank::Vector, "Divergences are only available for vector fields");
    return get_divergence<Rank>(field_index, type);
  }

  template <TensorRank Rank>
  PPF_HD ScalarValue get_divergence(unsigned int field_index, DependencyType type) const {
    const int row = row_of(field_index, type);
    ScalarValue s(number(0));
    if (row < 0) return s;
    for (int d = 0; d < int(dim); ++d) s += deriv(row + d, d);
    return s;
  }

  template <TensorRank Rank, DependencyType type>
  PPF_HD dealii::Tensor<1, (dim == 2 ? 1 : dim), ScalarValue> get_curl(unsigned int field_index) const {
    static_assert(Rank == TensorRank::Vector, "Curl is only available for vector fields");
    return get_curl<Rank>(field_index, type);
  }

  template <TensorRank Rank>
  PPF_HD dealii::Tensor<1, (dim == 2 ? 1 : dim), ScalarValue> get_curl(unsigned int field_index,
                                                                      DependencyType type) const {
    const Gradient<Rank> g = get_gradient<Rank>(field_index, type);
    dealii::Tensor<1, (dim == 2 ? 1 : dim), ScalarValue> c;
    if constexpr (dim == 2) {
      c[0] = g[1][0] - g[0][1];
    } else if constexpr (dim == 3) {
      c[0] = g[2][1] - g[1][2];
      c[1] = g[0][2] - g[2][0];
      c[2] = g[1][0] - g[0][1];
    }
    return c;
  }

  // --- second derivatives -------------------------------------------------------------
  template <TensorRank Rank, DependencyType type>
  PPF_HD Hessian<Rank> get_hessian(unsigned int field_index) const { return get_hessian<Rank>(field_index, type); }

  template <TensorRank Rank>
  PPF_HD Hessian<Rank> get_hessian(unsigned int field_index, DependencyType type) const {
    const int row = row_of(field_index, type);
    Hessian<Rank> H;
    if (row < 0) return H;
    if constexpr (Rank == TensorRank::Scalar) {
      for (int d = 0; d < int(dim); ++d)
        for (int e = d; e < int(dim); ++e) {
          ScalarValue v = second(row, d, e);
          H[d][e] = v;
          H[e][d] = v;
        }
    } else {
      for (int c = 0; c < int(dim); ++c)
        for (int d = 0; d < int(dim); ++d)
          for (int e = d; e < int(dim); ++e) {
            ScalarValue v = second(row + c, d, e);
            H[c][d][e] = v;
            H[c][e][d] = v;
          }
    }
    return H;
  }

  template <TensorRank Rank, DependencyType type>
  PPF_HD Gradient<Rank> get_hessian_diagonal(unsigned int field_index) const {
    return get_hessian_diagonal<Rank>(field_index, type);
  }

  template <TensorRank Rank>
  PPF_HD Gradient<Rank> get_hessian_diagonal(unsigned int field_index, DependencyType type) const {
    const int row = row_of(field_index, type);
    Gradient<Rank> g;
    if (row < 0) return g;
    if constexpr (Rank == TensorRank::Scalar) {
      for (int d = 0; d < int(dim); ++d) g[d] = second(row, d, d);
    } else {
      for (int c = 0; c < int(dim); ++c)
        for (int d = 0; d < int(dim); ++d) g[c][d] = second(row + c, d, d);
    }
    return g;
  }

  template <TensorRank Rank, DependencyType type>
  PPF_HD Value<Rank> get_laplacian(unsigned int field_index) const { return get_laplacian<Rank>(field_index, type); }

  template <TensorRank Rank>
  PPF_HD Value<Rank> get_laplacian(unsigned int field_index, DependencyType type) const {
    const int row = row_of(field_index, type);
    if constexpr (Rank == TensorRank::Scalar || dim == 1) {
      ScalarValue s(number(0));
      if (row < 0) return s;
      for (int d = 0; d < int(dim); ++d) s += second(row, d, d);
      return s;
    } else {
      Value<Rank> v;
      if (row < 0) return v;
      for (int c = 0; c < int(dim); ++c) {
        ScalarValue s(number(0));
        for (int d = 0; d < int(dim); ++d) s += second(row + c, d, d);
        v[c] = s;
      }
      return v;
    }
  }

  // --- geometry -----------------------------------------------------------------------
  PPF_HD dealii::Point<dim, ScalarValue> get_q_point_location() const {
    dealii::Point<dim, ScalarValue> p;
    int qq = ctx.q;
    for (int d = 0; d < int(dim); ++d) {
      const int a = qq % n;
      qq /= n;
      p[d] = ctx.tab->lo[d] + (number(ctx.cell[d]) + ctx.tab->gl_x[a]) * ctx.tab->h[d];
    }
    return p;
  }

  PPF_HD ScalarValue get_element_volume() const { return ScalarValue(ctx.tab->vol); }

  // --- submissions --------------------------------------------------------------------
  PPF_HD void set_value_term(unsigned int field_index, const ScalarValue& val) {
    const int o = out_row(field_index);
    if (o < 0) return;
    ctx.outs[o * ctx.stride + slot()] = (ctx.lean || ctx.raw_values) ? val.v : val.v * ctx.tab->jxw[ctx.q];
    ctx.submitted |= 1 << (2 * ctx.tab->out_of[field_index]);
  }

  PPF_HD void set_value_term(unsigned int field_index, const dealii::Tensor<1, dim, ScalarValue>& val) {
    const int o = out_row(field_index);
    if (o < 0) return;
    for (int c = 0; c < int(dim); ++c)
      ctx.outs[(o + c * (1 + dim)) * ctx.stride + slot()] =
          (ctx.lean || ctx.raw_values) ? val[c].v : val[c].v * ctx.tab->jxw[ctx.q];
    ctx.submitted |= 1 << (2 * ctx.tab->out_of[field_index]);
  }

  PPF_HD void set_gradient_term(unsigned int field_index, const dealii::Tensor<1, dim, ScalarValue>& g) {
    const int o = out_row(field_index);
    if (o < 0) return;
    // gradients are stored unscaled: the integration weights (jdt) carry JxW / h_d
    for (int d = 0; d < int(dim); ++d) ctx.outs[(o + 1 + d) * ctx.stride + slot()] = g[d].v;
    ctx.submitted |= 2 << (2 * ctx.tab->out_of[field_index]);
  }

  PPF_HD void set_gradient_term(unsigned int field_index, const dealii::Tensor<2, dim, ScalarValue>& g) {
    const int o = out_row(field_index);
    if (o < 0) return;
    for (int c = 0; c < int(dim); ++c)
      for (int d = 0; d < int(dim); ++d)
        ctx.outs[(o + c * (1 + dim) + 1 + d) * ctx.stride + slot()] = g[c][d].v;
    ctx.submitted |= 2 << (2 * ctx.tab->out_of[field_index]);
  }

  PPF_HD void set_gradient_term(unsigned int field_index, const dealii::SymmetricTensor<2, dim, ScalarValue>& g) {
    set_gradient_term(field_index, dealii::Tensor<2, dim, ScalarValue>(g));
  }

 private:
  Ctx& ctx;

  // offset of point p of this thread's cell within a row
  PPF_HD int pt(int p) const { return ctx.cpt ? p * ctx.cpt + ctx.lc : ctx.lc * int(dofs_per_component) + p; }
  PPF_HD int slot() const { return pt(ctx.q); }

  PPF_HD int row_of(unsigned int field_index, DependencyType type) const {
    const int age = gpu::age_of(type);
    int s = -1;
    if (field_index < unsigned(gpu::MAX_FIELDS) && age >= 0) s = ctx.tab->slot_of[field_index][age];
    if (s < 0) {
#ifdef __CUDA_ARCH__
      atomicOr(ctx.err, int(gpu::ERR_UNDECLARED_DEPENDENCY));
#endif
      return -1;
    }
    return ctx.tab->slot_comp0[s];
  }

  PPF_HD int out_row(unsigned int field_index) const {
    int o = field_index < unsigned(gpu::MAX_FIELDS) ? ctx.tab->out_of[field_index] : -1;
    if (o < 0) {
#ifdef __CUDA_ARCH__
      atomicOr(ctx.err, int(gpu::ERR_UNDECLARED_SUBMISSION));
#endif
      return -1;
    }
    return ctx.tab->out_row0[o];
  }

  PPF_HD number nodal(int row, int q) const {
    if constexpr (std::is_same<number, double>::value && degree <= 2) {
      if (ctx.lean) {
        // the lane kernel: the row's double copy, or for a row read only as a gradient its
        // value rebuilt from the fixed-point copy (exact to 2^-58 of the cell's largest value)
        const int vs = ctx.tab->lane_vslot[row];
        if (vs >= 0) return ctx.vals[vs * ctx.stride + pt(q)];
        const int E = ctx.ex_in[row * ctx.cpb + ctx.lc];
        const long long x = ctx.vals_fx[ctx.tab->lane_gslot[row] * ctx.stride + pt(q)];
        const double v = gpu::fx::to_double_fast(x, E - 1023 - gpu::fx::TOP_VALUES, 1ull << 63, false);
        return E == gpu::fx::EXP_NONFINITE ? gpu::fx::quiet_nan() : v;
      }
    }
    return ctx.vals[row * ctx.stride + pt(q)];
  }
  // the row's first entry in the double copies (the lane kernel's slot, else the row itself)
  PPF_HD int vrow(int row) const {
    if constexpr (std::is_same<number, double>::value && degree <= 2) {
      if (ctx.lean) return ctx.tab->lane_vslot[row];
    }
    return row;
  }

  // first derivative along direction d at this thread's quadrature point
  PPF_HD number deriv(int row, int d) const {
    int stride_d = 1;
    for (int e = 0; e < d; ++e) stride_d *= n;
    if constexpr (std::is_same<number, double>::value && degree <= 2) {
      if (ctx.lean && ((ctx.tab->fx_rows >> row) & 1u)) {
        // the lane kernel (rows read as gradients have a fixed-point copy; the test is uniform):
        // the line's fixed-point values at a point stride of cpt, the exact sum for this point's
        // position qd on the line, rounded once with 1/h_d folded in; NaN for a cell holding a
        // non-finite value (block exponent 2047)
        const int qd = ctx.qi[d];
        const int E = ctx.ex_in[row * ctx.cpb + ctx.lc];
        const int sq = stride_d * ctx.cpt;
        const long long* u =
            ctx.vals_fx + ctx.tab->lane_gslot[row] * ctx.stride + (ctx.q - qd * stride_d) * ctx.cpt + ctx.lc;
        long long s;
        if constexpr (n == 2) {
          s = u[sq] - u[0];
        } else {
          const long long u0 = u[0], u2 = u[2 * sq];
          const long long a = u2 - u0;
          const long long b = (u0 + u2 - (u[sq] << 1)) << 1;
          s = qd == 1 ? a : (qd == 0 ? a - b : a + b);
        }
        const double g = gpu::fx::to_double_fast(s, E - 1023 - gpu::fx::TOP_VALUES + ctx.tab->dk[d],
                                                 ctx.tab->dsig[d], ctx.tab->dpow2[d] == 0);
        return E == gpu::fx::EXP_NONFINITE ? gpu::fx::quiet_nan() : g;
      }
    }
    const int qd = (ctx.q / stride_d) % n;
    const int base = row * ctx.stride + ctx.lc * int(dofs_per_component) + (ctx.q - qd * stride_d);
    if constexpr (std::is_same<number, double>::value && degree <= 2) {
      if (ctx.vals_fx && !ctx.lean) {
        // exact integer sum of the line's fixed-point values, rounded once (1/h_d folded in)
        const int E = ctx.ex_in[row * ctx.cpb + ctx.lc];
        if (E == gpu::fx::EXP_NONFINITE) return gpu::fx::quiet_nan();
        if (E >= 0) {
        const long long* u = ctx.vals_fx + base;
        const long long s =
            gpu::fx::line_derivative<n>(qd, u[0], u[stride_d], n > 2 ? u[2 * stride_d] : 0ll);
        return gpu::fx::to_double(s, E - 1023 - gpu::fx::TOP_VALUES + ctx.tab->dk[d], ctx.tab->dsig[d]);
        }
        // a row declared without gradients has no fixed-point copy (exponent -1)
      }
    }
    // FP64 contraction over the nodal values
    const int q0 = ctx.q - qd * stride_d;
    const number* Dr = ctx.tab->Dh[d][qd];
    if (ctx.cpt) {
      const number* u = ctx.vals + vrow(row) * ctx.stride + q0 * ctx.cpt + ctx.lc;
      number s = Dr[0] * u[0];
#pragma unroll
      for (int j = 1; j < n; ++j) s = fma(Dr[j], u[j * stride_d * ctx.cpt], s);
      return s;
    }
    const number* u = ctx.vals + base;
    number s = Dr[0] * u[0];
#pragma unroll
    for (int j = 1; j < n; ++j) s = fma(Dr[j], u[j * stride_d], s);
    return s;
  }

  // second derivative d/dx_d d/dx_e at this thread's quadrature point
  PPF_HD number second(int row, int d, int e) const {
    int sd = 1, se = 1;
    for (int k = 0; k < d; ++k) sd *= n;
    for (int k = 0; k < e; ++k) se *= n;
    const int qd = (ctx.q / sd) % n, qe = (ctx.q / se) % n;
    const int vr = vrow(row);
    if (vr < 0) {
      // the lane kernel keeps no double copy of a row declared without values or Hessians
#ifdef __CUDA_ARCH__
      atomicOr(ctx.err, int(gpu::ERR_UNDECLARED_DEPENDENCY));
#endif
      return number(0);
    }
    const number* base = ctx.vals + vr * ctx.stride;
    if (d == e) {
      const int q0 = ctx.q - qd * sd;
      const number* Dr = ctx.tab->D2h[d][qd];
      number s = 0;
      for (int j = 0; j < n; ++j) s = fma(Dr[j], base[pt(q0 + j * sd)], s);
      return s;
    }
    const int q0 = ctx.q - qd * sd - qe * se;
    number s = 0;
    for (int j = 0; j < n; ++j) {
      number t = 0;
      for (int k = 0; k < n; ++k) t = fma(ctx.tab->Dh[e][qe][k], base[pt(q0 + j * sd + k * se)], t);
      s = fma(ctx.tab->Dh[d][qd][j], t, s);
    }
    return s;
  }
};

PRISMS_PF_END_NAMESPACE
