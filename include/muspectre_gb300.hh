/*
 * muspectre_gb300.hh -- C++ API of the GB300 Newton-CG path, with µSpectre's names.
 *
 * Header-only layer over the C ABI of musg.h (link with libmusg.so).  Namespace
 * muSpectre::gpu mirrors the reference's C++ interface for this path:
 *   make_cell<Dim>(res, lengths, form) / CellBase<Dim>      cell_factory.hh:93-105, cell_base.hh:70-526
 *   MaterialLinearElastic{1,2,3,4}<Dim>::make(cell, ...)    material_muSpectre_base.hh:135-137
 *   MaterialHyperElastoPlastic1<Dim>::make(cell, ...)       material_hyper_elasto_plastic1.hh
 *   MaterialLinearElasticGeneric<Dim>::make(cell, name, C_voigt)  material_linear_elastic_generic.hh
 *   SolverCG(cell, tol, maxiter, verbose)                   solver_cg.hh, solver_base.hh:62-109
 *   newton_cg(cell, load_steps, solver, newton_tol, equil_tol, verbose)  solvers.hh:54-74
 *   FFTEngine, ProjectionSmallStrain / ProjectionFiniteStrain(Fast)       fft_engine_base.hh, projection_*.hh
 *   ProjectionError, SolverError, ConvergenceError (std::runtime_error)  projection_base.hh, solver_common.hh
 * Vectors are std::vector<double> in the reference's layouts (see musg.h): a field
 * holds D*D doubles per pixel, column-major per pixel, pixels row-major.  Matrices
 * (loads, homogenised stress) are D*D column-major.  Materials are owned by their cell
 * and make() returns a reference, as in the reference.
 */
#ifndef MUSPECTRE_GB300_HH
#define MUSPECTRE_GB300_HH

#include <array>
#include <complex>
#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "musg.h"

namespace muSpectre {
namespace gpu {

using Real = double;
using Dim_t = int;
using Uint = unsigned int;

enum class Formulation { finite_strain = MUSG_FINITE_STRAIN, small_strain = MUSG_SMALL_STRAIN };
enum class FFT_PlanFlags { estimate = 0, measure = 1, patient = 2 };
enum class Precision { fp64 = MUSG_PRECISION_FP64, mixed = MUSG_PRECISION_MIXED };

struct ProjectionError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct SolverError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct ConvergenceError : SolverError {
  using SolverError::SolverError;
};
struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// maps a status code back onto the reference's exception types
inline void check(int rc) {
  if (rc == MUSG_OK) return;
  const std::string msg = musg_last_error();
  switch (rc) {
    case MUSG_ERR_PROJECTION: throw ProjectionError(msg);
    case MUSG_ERR_CONVERGENCE: throw ConvergenceError(msg);
    case MUSG_ERR_SOLVER: throw SolverError(msg);
    case MUSG_ERR_CUDA:
    case MUSG_ERR_MEMORY: throw CudaError(msg);
    case MUSG_ERR_ARGUMENT: throw std::invalid_argument(msg);
    default: throw std::runtime_error(msg);
  }
}

// OptimizeResult (solver_common.hh:50-67)
struct OptimizeResult {
  std::vector<Real> grad;
  std::vector<Real> stress;
  bool success = false;
  int status = 0;
  std::string message;
  Uint nb_it = 0;
  Uint nb_fev = 0;
};

class Cell;

// Communicator (src/common/communicator.hh:107-125, the build without MPI): one rank;
// a cell runs on one GPU, and independent cells on other GPUs need no exchange
class Communicator {
 public:
  int rank() const { return 0; }
  int size() const { return 1; }
  template <typename T> T sum(const T &arg) const { return arg; }
};

// MaterialBase (material_base.hh:103-150): a handle into the owning cell
class MaterialBase {
 public:
  MaterialBase(Cell &cell, int law, const std::string &name, const std::vector<Real> &params);
  virtual ~MaterialBase() = default;
  const std::string &get_name() const { return name_; }
  size_t size() const;
  int id() const { return id_; }

 protected:
  void add(const std::vector<long long> &pixels, const std::vector<Real> &per_pixel, int stride);
  long long index_of(const int *ccoord) const;
  Cell &cell_;
  std::string name_;
  int id_ = -1;
};

// Cell (cell_base.hh:115-233), the dimension-independent interface
class Cell {
 public:
  Cell(int dim, const int *res, const double *lengths, Formulation form, bool allow_even = false) : dim_(dim) {
    musg_cell *h = nullptr;
    check(musg_cell_create(dim, res, lengths, int(form), allow_even ? MUSG_FLAG_ALLOW_EVEN : 0, &h));
    h_ = h;
    form_ = form;
    for (int d = 0; d < dim; ++d) res_.push_back(res[d]);
  }
  Cell(const Cell &) = delete;
  Cell &operator=(const Cell &) = delete;
  virtual ~Cell() {
    if (h_) musg_cell_destroy(h_);
  }
  musg_cell *handle() const { return h_; }
  Dim_t get_dim() const { return dim_; }
  Dim_t get_nb_dof() const {
    long long n = 0;
    check(musg_cell_sizes(h_, &n, nullptr));
    return Dim_t(n);
  }
  size_t size() const {
    long long n = 0;
    check(musg_cell_sizes(h_, nullptr, &n));
    return size_t(n);
  }
  Formulation get_formulation() const { return form_; }
  // Cell::get_communicator (cell_base.hh:124, 502-503)
  const Communicator &get_communicator() const { return comm_; }
  std::array<Dim_t, 2> get_strain_shape() const { return {dim_, dim_}; }
  const std::vector<int> &get_domain_resolutions() const { return res_; }
  // CellBase::initialise (cell_base.cc:445-454)
  void initialise(FFT_PlanFlags flags = FFT_PlanFlags::estimate) { check(musg_cell_initialise(h_, int(flags))); }
  void set_uniform_strain(const std::vector<Real> &strain) { check(musg_cell_set_uniform_strain(h_, strain.data())); }
  std::vector<Real> get_strain_vector() {
    initialise();
    std::vector<Real> v(get_nb_dof());
    check(musg_cell_get_strain(h_, v.data()));
    return v;
  }
  void set_strain_vector(const std::vector<Real> &v) { check(musg_cell_set_strain(h_, v.data())); }
  std::vector<Real> get_stress_vector() {
    std::vector<Real> v(get_nb_dof());
    check(musg_cell_get_stress(h_, v.data()));
    return v;
  }
  // Cell::evaluate_stress_tangent (cell_base.cc:129-146): stress and tangent fields
  std::pair<std::vector<Real>, std::vector<Real>> evaluate_stress_tangent() {
    initialise();
    std::vector<Real> P(get_nb_dof()), K(size_t(get_nb_dof()) * dim_ * dim_);
    check(musg_cell_evaluate_stress_tangent(h_, P.data(), K.data()));
    return {std::move(P), std::move(K)};
  }
  std::vector<Real> evaluate_stress() {
    initialise();
    std::vector<Real> P(get_nb_dof());
    check(musg_cell_evaluate_stress_tangent(h_, P.data(), nullptr));
    return P;
  }
  // Cell::apply_projection (cell_base.cc:202-208), in place
  void apply_projection(std::vector<Real> &v) {
    initialise();
    check(musg_cell_apply_projection(h_, v.data()));
  }
  // Cell::evaluate_projected_directional_stiffness (cell_base.cc:150-192)
  std::vector<Real> evaluate_projected_directional_stiffness(const std::vector<Real> &dF) {
    std::vector<Real> out(get_nb_dof());
    check(musg_cell_directional_stiffness(h_, dF.data(), out.data()));
    return out;
  }
  void save_history_variables() { check(musg_cell_save_history_variables(h_)); }
  // CellBase::get_globalised_internal_real_array (cell_base.cc:370-436): values
  // pixel-major, nb_components per pixel
  std::vector<Real> get_globalised_internal_real_array(const std::string &name, int *nb_components = nullptr) {
    initialise();
    int nc = 0;
    check(musg_cell_get_internal(h_, name.c_str(), nullptr, 0, &nc));
    std::vector<Real> out(size() * size_t(nc));
    check(musg_cell_get_internal(h_, name.c_str(), out.data(), (long long)out.size(), &nc));
    if (nb_components) *nb_components = nc;
    return out;
  }
  // CellBase::get_managed_real_array (cell_base.cc:419-427): a cell-owned array of
  // nb_components values per pixel, created on first use
  std::vector<Real> &get_managed_real_array(const std::string &name, size_t nb_components) {
    auto it = managed_.find(name);
    if (it == managed_.end()) {
      managed_[name] = {nb_components, std::vector<Real>(nb_components * size(), 0.0)};
      return managed_[name].second;
    }
    if (it->second.first != nb_components)
      throw std::runtime_error("Field '" + name + "' already exists and it has " +
                               std::to_string(it->second.first) + " components. You asked for a field with " +
                               std::to_string(nb_components) + "components.");
    return it->second.second;
  }
  // extensions: homogenised stress (D*D column-major), checkpoint / restore
  std::vector<Real> homogenised_stress() {
    std::vector<Real> s(size_t(dim_) * dim_);
    check(musg_cell_homogenised_stress(h_, s.data()));
    return s;
  }
  std::vector<unsigned char> checkpoint() {
    unsigned long long n = 0;
    check(musg_cell_checkpoint_size(h_, &n));
    std::vector<unsigned char> img(n);
    check(musg_cell_checkpoint_save(h_, img.data(), n));
    return img;
  }
  void restore(const std::vector<unsigned char> &img) {
    check(musg_cell_checkpoint_load(h_, img.data(), img.size()));
  }
  // row-major linear pixel index of a ccoord (ccoord_operations.hh:179-192)
  long long get_index(const int *ccoord) const {
    long long idx = 0, f = 1;
    for (int d = dim_ - 1; d >= 0; --d) {
      idx += ccoord[d] * f;
      f *= res_[d];
    }
    return idx;
  }
  template <typename M> M &adopt(std::unique_ptr<M> m) {
    M &ref = *m;
    materials_.push_back(std::move(m));
    return ref;
  }

 protected:
  musg_cell *h_ = nullptr;
  int dim_ = 0;
  Formulation form_ = Formulation::finite_strain;
  std::vector<int> res_;
  std::vector<std::unique_ptr<MaterialBase>> materials_;
  std::map<std::string, std::pair<size_t, std::vector<Real>>> managed_;
  Communicator comm_;
};

// CellBase<DimS, DimM> with DimS = DimM = Dim
template <int Dim> class CellBase : public Cell {
 public:
  using Ccoord = std::array<int, Dim>;
  CellBase(const Ccoord &res, const std::array<Real, Dim> &lengths, Formulation form, bool allow_even = false)
      : Cell(Dim, res.data(), lengths.data(), form, allow_even) {}
  // ccoord of linear pixel i (ccoord_operations.hh:151-164); pixels run 0 .. size()-1
  Ccoord get_ccoord(size_t i) const {
    Ccoord c{};
    for (int d = Dim - 1; d >= 0; --d) {
      c[d] = int(i % size_t(res_[d]));
      i /= size_t(res_[d]);
    }
    return c;
  }
};

// make_cell<D, D>(res, lengths, form) (cell_factory.hh:93-105)
template <int Dim>
std::unique_ptr<CellBase<Dim>> make_cell(const std::array<int, Dim> &res, const std::array<Real, Dim> &lengths,
                                         Formulation form, bool allow_even = false) {
  return std::make_unique<CellBase<Dim>>(res, lengths, form, allow_even);
}

inline MaterialBase::MaterialBase(Cell &cell, int law, const std::string &name, const std::vector<Real> &params)
    : cell_(cell), name_(name) {
  check(musg_material_create(cell.handle(), law, name.c_str(), params.empty() ? nullptr : params.data(),
                             int(params.size()), &id_));
}
inline size_t MaterialBase::size() const {
  long long n = 0;
  check(musg_material_size(cell_.handle(), id_, &n));
  return size_t(n);
}
inline void MaterialBase::add(const std::vector<long long> &pixels, const std::vector<Real> &per_pixel, int stride) {
  check(musg_material_add_pixels(cell_.handle(), id_, pixels.data(), (long long)pixels.size(),
                                 per_pixel.empty() ? nullptr : per_pixel.data(), stride));
}
inline long long MaterialBase::index_of(const int *ccoord) const { return cell_.get_index(ccoord); }

// MaterialLinearElastic1 (material_linear_elastic1.hh:52-74)
template <int Dim> class MaterialLinearElastic1 : public MaterialBase {
 public:
  MaterialLinearElastic1(Cell &c, const std::string &name, Real young, Real poisson)
      : MaterialBase(c, MUSG_LAW_LE1, name, {young, poisson}) {}
  static MaterialLinearElastic1 &make(CellBase<Dim> &cell, const std::string &name, Real young, Real poisson) {
    return cell.adopt(std::make_unique<MaterialLinearElastic1>(cell, name, young, poisson));
  }
  void add_pixel(const std::array<int, Dim> &c) { add({index_of(c.data())}, {}, 0); }
  void add_pixels(const std::vector<long long> &idx) { add(idx, {}, 0); }
};

// MaterialLinearElastic2 (…elastic2.hh:179-201): per-pixel eigenstrain, D*D column-major
template <int Dim> class MaterialLinearElastic2 : public MaterialBase {
 public:
  MaterialLinearElastic2(Cell &c, const std::string &name, Real young, Real poisson)
      : MaterialBase(c, MUSG_LAW_LE2, name, {young, poisson}) {}
  static MaterialLinearElastic2 &make(CellBase<Dim> &cell, const std::string &name, Real young, Real poisson) {
    return cell.adopt(std::make_unique<MaterialLinearElastic2>(cell, name, young, poisson));
  }
  void add_pixel(const std::array<int, Dim> &c, const std::vector<Real> &eigenstrain) {
    add({index_of(c.data())}, eigenstrain, Dim * Dim);
  }
};

// MaterialLinearElastic3 / 4 (…elastic3.cc:58-68, …elastic4.cc:63-73): per-pixel (E, nu)
template <int Dim, int LAW> class MaterialLinearElasticPerPixel : public MaterialBase {
 public:
  MaterialLinearElasticPerPixel(Cell &c, const std::string &name) : MaterialBase(c, LAW, name, {}) {}
  static MaterialLinearElasticPerPixel &make(CellBase<Dim> &cell, const std::string &name) {
    return cell.adopt(std::make_unique<MaterialLinearElasticPerPixel>(cell, name));
  }
  void add_pixel(const std::array<int, Dim> &c, Real young, Real poisson) {
    add({index_of(c.data())}, {young, poisson}, 2);
  }
};
template <int Dim> using MaterialLinearElastic3 = MaterialLinearElasticPerPixel<Dim, MUSG_LAW_LE3>;
template <int Dim> using MaterialLinearElastic4 = MaterialLinearElasticPerPixel<Dim, MUSG_LAW_LE4>;

// MaterialLinearElasticGeneric (material_linear_elastic_generic.cc:40-66): a constant
// stiffness tensor from a Voigt matrix, vsize x vsize row-major (vsize 3 in 2-D, 6 in 3-D)
template <int Dim> class MaterialLinearElasticGeneric : public MaterialBase {
 public:
  MaterialLinearElasticGeneric(Cell &c, const std::string &name, const std::vector<Real> &C_voigt)
      : MaterialBase(c, MUSG_LAW_GENERIC, name, C_voigt) {}
  static MaterialLinearElasticGeneric &make(CellBase<Dim> &cell, const std::string &name,
                                           const std::vector<Real> &C_voigt) {
    return cell.adopt(std::make_unique<MaterialLinearElasticGeneric>(cell, name, C_voigt));
  }
  void add_pixel(const std::array<int, Dim> &c) { add({index_of(c.data())}, {}, 0); }
  void add_pixels(const std::vector<long long> &idx) { add(idx, {}, 0); }
};

// MaterialHyperElastoPlastic1 (material_hyper_elasto_plastic1.cc:41-65); mode 0 is the
// reference, 1 the spectral logm, 2 the spectral logm with the consistent tangent
// (extensions, see MUSG_LAW_HEP1)
template <int Dim> class MaterialHyperElastoPlastic1 : public MaterialBase {
 public:
  MaterialHyperElastoPlastic1(Cell &c, const std::string &name, Real young, Real poisson, Real tau_y0, Real H,
                              int mode = 0)
      : MaterialBase(c, MUSG_LAW_HEP1, name, {young, poisson, tau_y0, H, Real(mode)}) {}
  static MaterialHyperElastoPlastic1 &make(CellBase<Dim> &cell, const std::string &name, Real young, Real poisson,
                                          Real tau_y0, Real H, int mode = 0) {
    return cell.adopt(std::make_unique<MaterialHyperElastoPlastic1>(cell, name, young, poisson, tau_y0, H, mode));
  }
  void add_pixel(const std::array<int, Dim> &c) { add({index_of(c.data())}, {}, 0); }
};

// SolverBase / SolverCG (solver_base.hh:62-109, solver_cg.cc:54-110); Precision::mixed
// runs the inner CG in FP32 (an extension)
class SolverCG {
 public:
  SolverCG(Cell &cell, Real tol, Uint maxiter, bool verbose = false, Precision prec = Precision::fp64)
      : cell_(cell), tol_(tol), maxiter_(maxiter) {
    cell.initialise();
    check(musg_solver_cg_create(cell.handle(), tol, maxiter, verbose ? 1 : 0, int(prec), &h_));
  }
  SolverCG(const SolverCG &) = delete;
  SolverCG &operator=(const SolverCG &) = delete;
  ~SolverCG() {
    if (h_) musg_solver_destroy(h_);
  }
  musg_solver *handle() const { return h_; }
  void initialise() {}
  std::string get_name() const { return "CG"; }
  Real get_tol() const { return tol_; }
  Uint get_maxiter() const { return maxiter_; }
  Uint get_counter() const {
    unsigned c = 0;
    check(musg_solver_get_counter(h_, &c));
    return c;
  }
  void reset_counter() { check(musg_solver_reset_counter(h_)); }
  bool has_converged() const {
    int c = 0;
    check(musg_solver_has_converged(h_, &c));
    return c != 0;
  }
  void set_inner_tol(Real t) { check(musg_solver_set_inner_tol(h_, t)); }
  // newton_cg with a backtracking line search (extension; see musg_solver_set_line_search)
  void set_line_search(bool on) { check(musg_solver_set_line_search(h_, on ? 1 : 0)); }
  // mixed precision: FP32 corrections of the Newton residual (extension; see
  // musg_solver_set_incremental_residual)
  void set_incremental_residual(bool on) { check(musg_solver_set_incremental_residual(h_, on ? 1 : 0)); }
  // SolverCG::solve: x = A^-1 rhs
  std::vector<Real> solve(const std::vector<Real> &rhs) {
    std::vector<Real> x(rhs.size());
    check(musg_solver_solve(h_, rhs.data(), x.data()));
    return x;
  }
  Cell &get_cell() { return cell_; }

 private:
  Cell &cell_;
  musg_solver *h_ = nullptr;
  Real tol_;
  Uint maxiter_;
};

// newton_cg (solvers.cc:44-217): load_steps are D*D column-major macroscopic strains
inline std::vector<OptimizeResult> newton_cg(Cell &cell, const std::vector<std::vector<Real>> &load_steps,
                                             SolverCG &solver, Real newton_tol, Real equil_tol, Dim_t verbose = 0,
                                             bool return_fields = true) {
  const int D2 = cell.get_dim() * cell.get_dim();
  std::vector<Real> flat;
  for (const auto &s : load_steps) {
    if (int(s.size()) != D2)
      throw SolverError("Load increments need to be given in " + std::to_string(cell.get_dim()) + "×" +
                        std::to_string(cell.get_dim()) + " matrices");
    flat.insert(flat.end(), s.begin(), s.end());
  }
  const int n = int(load_steps.size());
  std::vector<musg_result_info> infos(n);
  const size_t nd = size_t(cell.get_nb_dof());
  std::vector<Real> grads(return_fields ? n * nd : 0), stresses(return_fields ? n * nd : 0);
  check(musg_newton_cg(cell.handle(), flat.data(), n, solver.handle(), newton_tol, equil_tol, verbose, infos.data(),
                       return_fields ? grads.data() : nullptr, return_fields ? stresses.data() : nullptr));
  std::vector<OptimizeResult> out(n);
  for (int k = 0; k < n; ++k) {
    out[k].success = infos[k].success != 0;
    out[k].status = infos[k].status;
    out[k].message = infos[k].message;
    out[k].nb_it = infos[k].nb_it;
    out[k].nb_fev = infos[k].nb_fev;
    if (return_fields) {
      out[k].grad.assign(grads.begin() + k * nd, grads.begin() + (k + 1) * nd);
      out[k].stress.assign(stresses.begin() + k * nd, stresses.begin() + (k + 1) * nd);
    }
  }
  return out;
}

// de_geus (solvers.cc:220-408), same arguments and results as newton_cg
inline std::vector<OptimizeResult> de_geus(Cell &cell, const std::vector<std::vector<Real>> &load_steps,
                                           SolverCG &solver, Real newton_tol, Real equil_tol, Dim_t verbose = 0) {
  const int D2 = cell.get_dim() * cell.get_dim();
  std::vector<Real> flat;
  for (const auto &s : load_steps) {
    if (int(s.size()) != D2) throw SolverError("Load increments need to be given in D×D matrices");
    flat.insert(flat.end(), s.begin(), s.end());
  }
  const int n = int(load_steps.size());
  std::vector<musg_result_info> infos(n);
  const size_t nd = size_t(cell.get_nb_dof());
  std::vector<Real> grads(n * nd), stresses(n * nd);
  check(musg_de_geus(cell.handle(), flat.data(), n, solver.handle(), newton_tol, equil_tol, verbose, infos.data(),
                     grads.data(), stresses.data()));
  std::vector<OptimizeResult> out(n);
  for (int k = 0; k < n; ++k) {
    out[k].success = infos[k].success != 0;
    out[k].status = infos[k].status;
    out[k].message = infos[k].message;
    out[k].nb_it = infos[k].nb_it;
    out[k].nb_fev = infos[k].nb_fev;
    out[k].grad.assign(grads.begin() + k * nd, grads.begin() + (k + 1) * nd);
    out[k].stress.assign(stresses.begin() + k * nd, stresses.begin() + (k + 1) * nd);
  }
  return out;
}

// the single-load overload (solvers.hh:65-74)
inline OptimizeResult newton_cg(Cell &cell, const std::vector<Real> &delF0, SolverCG &solver, Real newton_tol,
                                Real equil_tol, Dim_t verbose = 0) {
  return newton_cg(cell, std::vector<std::vector<Real>>{delF0}, solver, newton_tol, equil_tol, verbose)[0];
}

// FFTEngineBase (fft_engine_base.hh:75-148): unnormalised r2c / c2r of nb_components
// fields; the workspace holds nb_hermitian*nb_components complex values
class FFTEngine {
 public:
  FFTEngine(const std::vector<int> &res, int nb_components) : res_(res), nc_(nb_components) {
    check(musg_fft_create(int(res.size()), res.data(), nb_components, &h_));
  }
  ~FFTEngine() {
    if (h_) musg_fft_destroy(h_);
  }
  FFTEngine(const FFTEngine &) = delete;
  FFTEngine &operator=(const FFTEngine &) = delete;
  size_t nb_pixels() const {
    size_t n = 1;
    for (int r : res_) n *= size_t(r);
    return n;
  }
  size_t nb_hermitian() const { return nb_pixels() / size_t(res_.back()) * size_t(res_.back() / 2 + 1); }
  Real normalisation() const { return 1.0 / Real(nb_pixels()); }
  std::vector<std::complex<Real>> fft(const std::vector<Real> &field) {
    std::vector<std::complex<Real>> ws(nb_hermitian() * size_t(nc_));
    check(musg_fft_forward(h_, field.data(), reinterpret_cast<double *>(ws.data())));
    return ws;
  }
  std::vector<Real> ifft(const std::vector<std::complex<Real>> &ws) {
    std::vector<Real> field(nb_pixels() * size_t(nc_));
    check(musg_fft_inverse(h_, reinterpret_cast<const double *>(ws.data()), field.data()));
    return field;
  }

 private:
  std::vector<int> res_;
  int nc_;
  musg_fft *h_ = nullptr;
};

// ProjectionBase (projection_base.hh:99-161) and its three kinds
template <int KIND> class Projection {
 public:
  Projection(const std::vector<int> &res, const std::vector<Real> &lengths, bool allow_even = false) : res_(res) {
    check(musg_projection_create(int(res.size()), res.data(), lengths.data(), KIND,
                                 allow_even ? MUSG_FLAG_ALLOW_EVEN : 0, &h_));
  }
  ~Projection() {
    if (h_) musg_projection_destroy(h_);
  }
  Projection(const Projection &) = delete;
  Projection &operator=(const Projection &) = delete;
  void initialise(FFT_PlanFlags = FFT_PlanFlags::estimate) {}
  // in place on a field (D*D values per pixel)
  void apply_projection(std::vector<Real> &field) { check(musg_projection_apply(h_, field.data())); }
  Formulation get_formulation() const {
    return KIND == MUSG_PROJ_SMALL_STRAIN ? Formulation::small_strain : Formulation::finite_strain;
  }

 private:
  std::vector<int> res_;
  musg_projection *h_ = nullptr;
};
using ProjectionSmallStrain = Projection<MUSG_PROJ_SMALL_STRAIN>;
using ProjectionFiniteStrainFast = Projection<MUSG_PROJ_FINITE_STRAIN_FAST>;
using ProjectionFiniteStrain = Projection<MUSG_PROJ_FINITE_STRAIN>;

}  // namespace gpu
}  // namespace muSpectre

#endif  // MUSPECTRE_GB300_HH
