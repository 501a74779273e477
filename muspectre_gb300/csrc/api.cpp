// C ABI of libmusg (include/musg.h): cells, materials, SolverCG, newton_cg, the FFT
// engine and the projections.  Host C++ drives the device kernels; every field
// lives on the GPU and crosses to the host only at the API boundary (get_strain,
// get_stress, OptimizeResult copies).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "musg_internal.h"

using namespace musg;

namespace {

thread_local std::string g_last_error;

template <typename F> int guard(F &&f) {
  try {
    f();
    return MUSG_OK;
  } catch (const Error &e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    g_last_error = "host allocation failed";
    return MUSG_ERR_MEMORY;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return MUSG_ERR_RUNTIME;
  }
}

void require(bool ok, int code, const std::string &msg) {
  if (!ok) throw Error(code, msg);
}
// literal messages: no std::string is built unless the check fails (some checks run
// once per pixel)
void require(bool ok, int code, const char *msg) {
  if (!ok) throw Error(code, msg);
}

}  // namespace

int musg::guarded(const std::function<void()> &f) { return guard(f); }

namespace {

// Hooke helpers (src/materials/materials_toolbox.hh:491-525)
double lame_lambda(double E, double nu) { return E * nu / ((1 + nu) * (1 - 2 * nu)); }
double lame_mu(double E, double nu) { return E / (2 * (1 + nu)); }
double bulk_K(double E, double nu) { return E / (3 * (1 - 2 * nu)); }

std::string ccoord_str(const int *res, int dim, long long idx) {
  int c[3] = {0, 0, 0};
  for (int d = dim - 1; d >= 0; --d) {
    c[d] = (int)(idx % res[d]);
    idx /= res[d];
  }
  std::ostringstream o;
  o << "(";
  for (int d = 0; d < dim; ++d) o << (d ? ", " : "") << c[d];
  o << ")";
  return o.str();
}

// Launch shapes found by the autotuner, shared by every cell of the same grid,
// component count and projection in this process (cf. FFTW wisdom).
struct Wisdom {
  int threads[3];
  long bytes[3];
};
std::mutex g_wisdom_mu;
std::map<std::string, Wisdom> g_wisdom;

std::string wisdom_key(const Spectral &sp, int prec) {
  std::ostringstream k;
  k << sp.g.dim << ':' << sp.g.n[0] << 'x' << sp.g.n[1] << 'x' << sp.g.n[2] << ':' << sp.ncomp << ':'
    << sp.proj_kind << ':' << sp.allow_even << ':' << prec;
  return k.str();
}

template <typename R> void autotune_with_wisdom(Spectral &sp, cudaStream_t s, int effort) {
  const int pi = sizeof(R) == 8 ? 0 : 1;
  const std::string key = wisdom_key(sp, pi);
  {
    std::lock_guard<std::mutex> lock(g_wisdom_mu);
    auto it = g_wisdom.find(key);
    if (it != g_wisdom.end()) {
      for (int k = 0; k < 3; ++k) {
        sp.tune_threads[pi][k] = it->second.threads[k];
        sp.tune_bytes[pi][k] = it->second.bytes[k];
      }
      return;
    }
  }
  spectral_autotune<R>(sp, s, effort);
  Wisdom w;
  for (int k = 0; k < 3; ++k) {
    w.threads[k] = sp.tune_threads[pi][k];
    w.bytes[k] = sp.tune_bytes[pi][k];
  }
  std::lock_guard<std::mutex> lock(g_wisdom_mu);
  g_wisdom[key] = w;
}

struct Material {
  int law = 0;
  std::string name;
  double E = 0, nu = 0, tau_y0 = 0, H = 0;
  int logm_mode = 0;
  std::vector<long long> pixels;
  std::vector<double> per_pixel;  // stride values per pixel
  int stride = 0;
  std::vector<double> C;          // MaterialLinearElasticGeneric: D^4 stiffness (T4 layout)
};

// MaterialLinearElasticGeneric (material_linear_elastic_generic.cc:40-66): C(i,j,k,l) =
// C_voigt(sym(i,j), sym(k,l)) with the Voigt index map of voigt_conversion.hh:118-125
std::vector<double> stiffness_from_voigt(const double *voigt, int dim) {
  static const int sym2[2][2] = {{0, 2}, {2, 1}};
  static const int sym3[3][3] = {{0, 5, 4}, {5, 1, 3}, {4, 3, 2}};
  const int vs = dim == 2 ? 3 : 6, D2 = dim * dim;
  auto sym = [&](int i, int j) { return dim == 2 ? sym2[i][j] : sym3[i][j]; };
  std::vector<double> C((size_t)D2 * D2);
  for (int l = 0; l < dim; ++l)
    for (int k = 0; k < dim; ++k)
      for (int j = 0; j < dim; ++j)
        for (int i = 0; i < dim; ++i) C[(i + dim * j) + D2 * (k + dim * l)] = voigt[sym(i, j) * vs + sym(k, l)];
  return C;
}

// isotropic C = lam I (x) I + mu (I_sym doubled) (materials_toolbox.hh:638-652)
std::vector<double> stiffness_isotropic(double lam, double mu, int dim) {
  const int D2 = dim * dim;
  std::vector<double> C((size_t)D2 * D2);
  for (int l = 0; l < dim; ++l)
    for (int k = 0; k < dim; ++k)
      for (int j = 0; j < dim; ++j)
        for (int i = 0; i < dim; ++i)
          C[(i + dim * j) + D2 * (k + dim * l)] =
              (i == j && k == l ? lam : 0.0) + mu * ((i == k && j == l ? 1.0 : 0.0) + (i == l && j == k ? 1.0 : 0.0));
  return C;
}

}  // namespace

struct musg_cell {
  int dim = 0, form = 0, flags = 0;
  int res[3] = {1, 1, 1};
  double lengths[3] = {1, 1, 1};
  long long npx = 0;
  int D2 = 0;
  bool initialised = false;
  bool tangent_valid = false;
  bool need32 = false;
  int plan_flags = 0;      // FFT_PlanFlags: estimate 0, measure 1, patient 2
  bool tuned64 = false, tuned32 = false;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::vector<Material> materials;
  Spectral sp;
  int tkind = TK_SMALL, tkind32 = TK_SMALL;  // CG operator kind of the FP64 / FP32 path
  template <typename R> int tk() const { return sizeof(R) == 4 ? tkind32 : tkind; }
  int hep_cur = 0;
  bool has_le2 = false, has_hep = false;
  bool has_consistent = false;  // an HEP1 material with the consistent tangent: TK_FULL cell
  // device fields (FP64 component planes)
  DevBuf F, P, rhs, io, io2, F0;  // F0: the line search's Newton iterate
  DevBuf Pk, dP32;                // the stress of the last projected residual; FP32 projection input
  bool residual_kept = false;     // Pk and rhs belong together (incremental residual)
  DevBuf mat, params, law_kind, Ctab64, Ctab32;
  bool has_generic = false;
  DevBuf lam64, mu64, lam32, mu32, eig;
  DevBuf Fprev[2], be[2], eps[2];
  DevBuf S64, S32, Kp64, Kp32, Fc64, Fc32, Kfull, Kt64, Kt32;
  DevBuf partial, scal;  // reduction scratch, small device scalars
  DevBuf nonfinite;
  double *hscal = nullptr;  // pinned host mirror of scal

  ~musg_cell() {
    if (hscal) cudaFreeHost(hscal);
    sp.release();
    if (own_stream && stream) cudaStreamDestroy(stream);
  }
  long long nb_dof() const { return npx * D2; }
  size_t plane_bytes() const { return (size_t)npx * sizeof(double); }
  size_t field_bytes() const { return (size_t)nb_dof() * sizeof(double); }

  void create(int dim_, const int *res_, const double *len_, int form_, int flags_) {
    require(dim_ == 2 || dim_ == 3, MUSG_ERR_ARGUMENT, "only 2- and 3-dimensional cells are supported");
    require(form_ == MUSG_FINITE_STRAIN || form_ == MUSG_SMALL_STRAIN, MUSG_ERR_ARGUMENT, "unknow formulation");
    dim = dim_;
    form = form_;
    flags = flags_;
    npx = 1;
    for (int d = 0; d < dim; ++d) {
      require(res_[d] > 0, MUSG_ERR_ARGUMENT, "resolutions must be positive");
      res[d] = res_[d];
      lengths[d] = len_ ? len_[d] : 1.0;
      npx *= res[d];
    }
    D2 = dim * dim;
    // projections reject even grids (projection_small_strain.cc:46-51,
    // projection_finite_strain_fast.cc:50-55) unless the extension is asked for
    if (!(flags & MUSG_FLAG_ALLOW_EVEN))
      for (int d = 0; d < dim; ++d)
        require(res[d] % 2 == 1, MUSG_ERR_PROJECTION, "Only an odd number of gridpoints in each direction is supported");
    MUSG_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    own_stream = true;
    const int proj = form == MUSG_FINITE_STRAIN ? MUSG_PROJ_FINITE_STRAIN_FAST : MUSG_PROJ_SMALL_STRAIN;
    sp.init(dim, res, D2, proj, lengths, (flags & MUSG_FLAG_ALLOW_EVEN) != 0, false);
    F.alloc(field_bytes());
    P.alloc(field_bytes());
    rhs.alloc(field_bytes());
    MUSG_CUDA(cudaMemsetAsync(F.p, 0, field_bytes(), stream));
    MUSG_CUDA(cudaMemsetAsync(P.p, 0, field_bytes(), stream));
    // reduction scratch: block or per-warp partial sums of the passes (at most 16 warps
    // per half row pair of the last-axis passes)
    partial.alloc((size_t)std::max<long long>(4 * 4096, 16 * sp.g.nrows + 64) * sizeof(double));
    scal.alloc(64 * sizeof(double));
    nonfinite.alloc(sizeof(int));
    MUSG_CUDA(cudaMemsetAsync(nonfinite.p, 0, sizeof(int), stream));
    MUSG_CUDA(cudaMallocHost(&hscal, 64 * sizeof(double)));
    MUSG_CUDA(cudaStreamSynchronize(stream));
  }

  // device vector of D2 doubles (column-major matrix) into scal[off..]
  double *put_matrix(const double *m, int off) {
    for (int c = 0; c < D2; ++c) hscal[off + c] = m[c];
    MUSG_CUDA(cudaMemcpyAsync(scal.as<double>() + off, hscal + off, D2 * sizeof(double), cudaMemcpyHostToDevice, stream));
    MUSG_CUDA(cudaStreamSynchronize(stream));  // the pinned slot may be rewritten next
    return scal.as<double>() + off;
  }

  void check_material_coverage() {
    // cell_base.cc:486-526
    std::vector<int> owner(npx, -1);
    for (size_t m = 0; m < materials.size(); ++m)
      for (long long p : materials[m].pixels) {
        if (owner[p] != -1) {
          std::ostringstream e;
          e << "Pixel " << ccoord_str(res, dim, p) << "is already assigned to material '" << materials[owner[p]].name
            << "' and cannot be reassigned to material '" << materials[m].name;
          throw Error(MUSG_ERR_RUNTIME, e.str());
        }
        owner[p] = (int)m;
      }
    long long missing = 0;
    std::ostringstream e;
    e << "The following pixels have were not assigned a material: ";
    for (long long p = 0; p < npx; ++p)
      if (owner[p] < 0) {
        if (missing < 16) e << ccoord_str(res, dim, p) << ", ";
        ++missing;
      }
    if (missing) {
      if (missing > 16) e << "... (" << missing << " pixels), ";
      e << "and that cannot be handled";
      throw Error(MUSG_ERR_RUNTIME, e.str());
    }
  }

  void initialise() {
    if (initialised) return;
    require(!materials.empty(), MUSG_ERR_RUNTIME, "no materials in the cell");
    require(materials.size() <= (size_t)kMaxMaterials, MUSG_ERR_ARGUMENT, "at most 256 materials per cell");
    check_material_coverage();
    std::vector<uint8_t> hmat(npx);
    // per-pixel Lame constants on the host only for the laws that have them per pixel;
    // the others are filled on the device from the material index
    bool per_pixel_lame = false;
    for (const Material &mt : materials) per_pixel_lame |= mt.law == MUSG_LAW_LE3 || mt.law == MUSG_LAW_LE4;
    std::vector<double> hlam(per_pixel_lame ? npx : 0), hmu(per_pixel_lame ? npx : 0);
    std::vector<MatParams> hp(materials.size());
    std::vector<uint8_t> hkind(kMaxMaterials, TK_FINITE);
    bool any_le = false;
    for (size_t m = 0; m < materials.size(); ++m) {
      const Material &mt = materials[m];
      MatParams &q = hp[m];
      q.law = mt.law;
      q.logm_mode = mt.logm_mode;
      q.lam = lame_lambda(mt.E, mt.nu);
      q.mu = lame_mu(mt.E, mt.nu);
      q.K = bulk_K(mt.E, mt.nu);
      q.tau_y0 = mt.tau_y0;
      q.H = mt.H;
      if (mt.law == MUSG_LAW_HEP1) {
        has_hep = true;
        has_consistent |= mt.logm_mode == kHep1Consistent;
        hkind[m] = TK_KPRIME;
      } else {
        any_le = true;
      }
      if (mt.law == MUSG_LAW_LE2) has_le2 = true;
      if (mt.law == MUSG_LAW_GENERIC) has_generic = true;
      for (size_t k = 0; k < mt.pixels.size(); ++k) {
        const long long p = mt.pixels[k];
        hmat[p] = (uint8_t)m;
        if (!per_pixel_lame) continue;
        if (mt.law == MUSG_LAW_LE3 || mt.law == MUSG_LAW_LE4) {
          const double E = mt.per_pixel[2 * k], nu = mt.per_pixel[2 * k + 1];
          hlam[p] = lame_lambda(E, nu);
          hmu[p] = lame_mu(E, nu);
        } else {
          hlam[p] = q.lam;
          hmu[p] = q.mu;
        }
      }
    }
    require(!(has_hep && form == MUSG_SMALL_STRAIN), MUSG_ERR_ARGUMENT,
            "MaterialHyperElastoPlastic1 needs the finite-strain formulation");
    if (form == MUSG_SMALL_STRAIN) tkind = TK_SMALL;
    else if (has_consistent) tkind = TK_FULL;  // every pixel's dP/dF stored (D^4 planes)
    else if (has_hep && any_le) tkind = TK_MIXED;
    else if (has_hep) tkind = TK_KPRIME;
    else tkind = TK_FINITE;
    if (has_generic) {
      // per-material stiffness tables: every material of the cell has a constant C
      for (const Material &mt : materials)
        require(mt.law == MUSG_LAW_LE1 || mt.law == MUSG_LAW_LE2 || mt.law == MUSG_LAW_GENERIC, MUSG_ERR_ARGUMENT,
                "MaterialLinearElasticGeneric shares a cell with LE1, LE2 and generic materials only");
      tkind = form == MUSG_SMALL_STRAIN ? TK_GSMALL : TK_GFINITE;
      std::vector<double> ct;
      for (size_t m = 0; m < materials.size(); ++m) {
        const std::vector<double> Cm = materials[m].law == MUSG_LAW_GENERIC
                                           ? materials[m].C
                                           : stiffness_isotropic(hp[m].lam, hp[m].mu, dim);
        ct.insert(ct.end(), Cm.begin(), Cm.end());
      }
      std::vector<float> cf(ct.begin(), ct.end());
      Ctab64.alloc(ct.size() * sizeof(double));
      Ctab32.alloc(cf.size() * sizeof(float));
      MUSG_CUDA(cudaMemcpy(Ctab64.p, ct.data(), Ctab64.bytes, cudaMemcpyHostToDevice));
      MUSG_CUDA(cudaMemcpy(Ctab32.p, cf.data(), Ctab32.bytes, cudaMemcpyHostToDevice));
    }
    // the FP32 operator rebuilds S from F where the law allows (not LE2: eigenstrain)
    tkind32 = (tkind == TK_FINITE && !has_le2) ? TK_FISO : tkind;
    mat.alloc(npx);
    MUSG_CUDA(cudaMemcpy(mat.p, hmat.data(), npx, cudaMemcpyHostToDevice));
    params.alloc(hp.size() * sizeof(MatParams));
    MUSG_CUDA(cudaMemcpy(params.p, hp.data(), hp.size() * sizeof(MatParams), cudaMemcpyHostToDevice));
    law_kind.alloc(kMaxMaterials);
    MUSG_CUDA(cudaMemcpy(law_kind.p, hkind.data(), kMaxMaterials, cudaMemcpyHostToDevice));
    lam64.alloc(plane_bytes());
    mu64.alloc(plane_bytes());
    if (per_pixel_lame) {
      MUSG_CUDA(cudaMemcpy(lam64.p, hlam.data(), plane_bytes(), cudaMemcpyHostToDevice));
      MUSG_CUDA(cudaMemcpy(mu64.p, hmu.data(), plane_bytes(), cudaMemcpyHostToDevice));
    } else {
      fill_lame(mat.as<uint8_t>(), params.as<MatParams>(), lam64.as<double>(), mu64.as<double>(), npx, stream);
    }
    if (has_le2) {
      std::vector<double> h((size_t)npx * D2, 0.0);
      for (const Material &mt : materials)
        if (mt.law == MUSG_LAW_LE2)
          for (size_t k = 0; k < mt.pixels.size(); ++k)
            for (int c = 0; c < D2; ++c) h[(size_t)c * npx + mt.pixels[k]] = mt.per_pixel[k * D2 + c];
      eig.alloc(field_bytes());
      MUSG_CUDA(cudaMemcpy(eig.p, h.data(), field_bytes(), cudaMemcpyHostToDevice));
    }
    if (form == MUSG_FINITE_STRAIN) {
      S64.alloc(field_bytes());
      Fc64.alloc(field_bytes());  // F at the last evaluation (the tangent's F)
    }
    if (has_hep) {
      // material_hyper_elasto_plastic1.cc:76-84: zero-initialised state fields,
      // current() of F_prev and b_e set to I, then one cycle
      for (int b = 0; b < 2; ++b) {
        Fprev[b].alloc(field_bytes());
        be[b].alloc(field_bytes());
        eps[b].alloc(plane_bytes());
        MUSG_CUDA(cudaMemset(Fprev[b].p, 0, field_bytes()));
        MUSG_CUDA(cudaMemset(be[b].p, 0, field_bytes()));
        MUSG_CUDA(cudaMemset(eps[b].p, 0, plane_bytes()));
      }
      std::vector<double> I(D2, 0.0);
      for (int i = 0; i < dim; ++i) I[i + dim * i] = 1.0;
      double *Id = put_matrix(I.data(), 0);
      fill_uniform(Fprev[0].as<double>(), Id, D2, npx, stream);
      fill_uniform(be[0].as<double>(), Id, D2, npx, stream);
      hep_cur = 1;
      if (tkind == TK_FULL) Kt64.alloc((size_t)npx * D2 * D2 * sizeof(double));
      else Kp64.alloc((size_t)npx * D2 * dim * sizeof(double));
    }
    if (need32) alloc32();
    initialised = true;
    autotune();
    MUSG_CUDA(cudaStreamSynchronize(stream));
  }

  // FFT_PlanFlags::measure / patient: time the launch shapes of the passes on this
  // grid (the analogue of FFTW planning with FFTW_MEASURE)
  void autotune() {
    if (plan_flags < 1 || !initialised) return;
    if (!tuned64) {
      autotune_with_wisdom<double>(sp, stream, plan_flags);
      tuned64 = true;
    }
    if (need32 && !tuned32) {
      autotune_with_wisdom<float>(sp, stream, plan_flags);
      tuned32 = true;
    }
  }

  void alloc32() {
    need32 = true;
    sp.ensure32();
    if (!initialised && !lam64.p) return;  // done at initialise
    if (!lam32.p) {
      lam32.alloc((size_t)npx * sizeof(float));
      mu32.alloc((size_t)npx * sizeof(float));
      convert<float, double>(lam32.as<float>(), lam64.as<double>(), npx, 1.0, stream);
      convert<float, double>(mu32.as<float>(), mu64.as<double>(), npx, 1.0, stream);
    }
    if (form == MUSG_FINITE_STRAIN) {
      if (!S32.p) S32.alloc((size_t)nb_dof() * sizeof(float));
      if (!Fc32.p) Fc32.alloc((size_t)nb_dof() * sizeof(float));
      if (has_hep && tkind != TK_FULL && !Kp32.p) Kp32.alloc((size_t)npx * D2 * dim * sizeof(float));
      if (tkind == TK_FULL && !Kt32.p) Kt32.alloc((size_t)npx * D2 * D2 * sizeof(float));
    }
    tangent_valid = false;
    autotune();
  }

  void evaluate(bool want_K) {
    if (!initialised) initialise();
    MaterialArgs a{};
    a.dim = dim;
    a.form = form;
    a.npx = npx;
    a.F = F.as<double>();
    a.P = P.as<double>();
    a.mat = mat.as<uint8_t>();
    a.params = params.as<MatParams>();
    a.lam = lam64.as<double>();
    a.mu = mu64.as<double>();
    a.eig = has_le2 ? eig.as<double>() : nullptr;
    a.Ctab = Ctab64.as<double>();
    for (int b = 0; b < 2; ++b) {
      a.Fprev[b] = Fprev[b].as<double>();
      a.be[b] = be[b].as<double>();
      a.eps[b] = eps[b].as<double>();
    }
    a.cur = hep_cur;
    a.S64 = S64.as<double>();
    a.Kp64 = Kp64.as<double>();
    a.S32 = tkind32 == TK_FISO ? nullptr : S32.as<float>();
    a.Kp32 = Kp32.as<float>();
    a.Kt64 = Kt64.as<double>();
    a.Kt32 = Kt32.as<float>();
    a.Fc32 = Fc32.as<float>();
    a.Fc64 = Fc64.as<double>();
    if (want_K) {
      if (Kfull.bytes < (size_t)nb_dof() * D2 * sizeof(double)) Kfull.alloc((size_t)nb_dof() * D2 * sizeof(double));
      a.Kfull = Kfull.as<double>();
    }
    a.nonfinite = nonfinite.as<int>();
    a.has_hep = has_hep ? 1 : 0;
    material_evaluate(a, stream);
    tangent_valid = true;
  }

  template <typename R> TangentData<R> tangent() const;

  void save_history() {
    // StateField::cycle (statefield.hh:322-326): swap current and old
    if (has_hep) hep_cur = 1 - hep_cur;
  }

  // the pixel mean of the stress field (D*D column-major) into out (host, 9 entries),
  // reduced on the device in a fixed order
  void homogenised(double *out) {
    double *d = scal.as<double>() + 40;
    plane_means(P.as<double>(), D2, npx, partial.as<double>(), d, stream);
    MUSG_CUDA(cudaMemcpyAsync(hscal + 40, d, D2 * sizeof(double), cudaMemcpyDeviceToHost, stream));
    MUSG_CUDA(cudaStreamSynchronize(stream));
    for (int k = 0; k < 9; ++k) out[k] = k < D2 ? hscal[40 + k] : 0.0;
  }

  // rhs = -G(P) for the current stress.  Incremental (the mixed path's default): the
  // first residual after residual_kept is cleared is projected in FP64 and its P kept
  // in Pk; each later one is G(rhs - (P - Pk)) projected in FP32 (rhs is in the range
  // of G, so this is rhs - G(P - Pk) = -G(P)), and the new P is kept.  The FP32
  // input is the previous residual minus the stress change since, whose size
  // shrinks with the Newton increments: the result carries FP32 rounding of that
  // change (not of P, whose mean and fluctuation are far larger), its part outside
  // the range of G is rounding of the result itself (the fused CG iteration needs
  // the right-hand side in that range), and the FP64 projections, bound by the FP64
  // pipe, drop to one per load step.
  void project_residual(bool incremental) {
    if (!incremental || !residual_kept) {
      spectral_project<double>(sp, P.as<double>(), rhs.as<double>(), -1.0, stream);
      if (incremental) {
        if (Pk.bytes < field_bytes()) Pk.alloc(field_bytes());
        MUSG_CUDA(cudaMemcpyAsync(Pk.p, P.p, field_bytes(), cudaMemcpyDeviceToDevice, stream));
        residual_kept = true;
      }
      return;
    }
    const long long n = nb_dof();
    if (dP32.bytes < (size_t)n * sizeof(float)) dP32.alloc((size_t)n * sizeof(float));
    residual_input(rhs.as<double>(), P.as<double>(), Pk.as<double>(), dP32.as<float>(), n, stream);
    spectral_project<float>(sp, dP32.as<float>(), dP32.as<float>(), 1.0f, stream);
    convert<double, float>(rhs.as<double>(), dP32.as<float>(), n, 1.0, stream);
  }

  // host AoS vector -> device SoA planes (dst)
  void upload_field(const double *host, double *dst) {
    if (io.bytes < field_bytes()) io.alloc(field_bytes());
    MUSG_CUDA(cudaMemcpyAsync(io.p, host, field_bytes(), cudaMemcpyHostToDevice, stream));
    aos_to_soa(io.as<double>(), dst, D2, npx, stream);
  }
  void download_field(const double *src, double *host) {
    if (io.bytes < field_bytes()) io.alloc(field_bytes());
    soa_to_aos(src, io.as<double>(), D2, npx, stream);
    MUSG_CUDA(cudaMemcpyAsync(host, io.p, field_bytes(), cudaMemcpyDeviceToHost, stream));
    MUSG_CUDA(cudaStreamSynchronize(stream));
  }
};

template <> TangentData<double> musg_cell::tangent<double>() const {
  TangentData<double> t;
  t.lam = lam64.as<double>();
  t.mu = mu64.as<double>();
  t.F = Fc64.as<double>();
  t.S = S64.as<double>();
  t.Kp = Kp64.as<double>();
  t.Kt = Kt64.as<double>();
  t.mat = mat.as<uint8_t>();
  t.law_kind = law_kind.as<uint8_t>();
  t.C = Ctab64.as<double>();
  return t;
}

template <> TangentData<float> musg_cell::tangent<float>() const {
  TangentData<float> t;
  t.lam = lam32.as<float>();
  t.mu = mu32.as<float>();
  t.F = Fc32.as<float>();
  t.S = S32.as<float>();
  t.Kp = Kp32.as<float>();
  t.Kt = Kt32.as<float>();
  t.mat = mat.as<uint8_t>();
  t.law_kind = law_kind.as<uint8_t>();
  t.C = Ctab32.as<float>();
  return t;
}

// ---------------------------------------------------------------------- solver
struct musg_solver {
  musg_cell *cell = nullptr;
  double tol = 0;
  unsigned maxiter = 0;
  int verbose = 0;
  int precision = MUSG_PRECISION_FP64;
  bool converged = false;
  unsigned long long counter = 0;
  DevBuf x, r, p, Ap, st;
  CGState *hst = nullptr;
  cudaGraphExec_t exec = nullptr;
  unsigned long long graph_nodes = 0;
  int chunk = 16;
  bool graphs = true;
  // mixed precision: the FP32 inner solve stops at max(tol, inner_tol), a forcing
  // term of inexact Newton (Eisenstat & Walker): each Newton step contracts the error
  // by about inner_tol and the FP64 Newton loop refines to newton_tol, so a loose
  // inner solve costs fewer CG iterations in total (FP32 CG could not go much below
  // ~1e-6 on stiff-contrast cells anyway)
  double inner_tol = 1e-2;
  // newton_cg with a backtracking line search on the projected residual norm (an
  // extension, off by default; needed by the consistent elasto-plastic tangent)
  bool line_search = false;
  // mixed precision: the Newton residual by FP32 corrections after one FP64 projection
  // per load step (musg_cell::project_residual)
  bool incremental_residual = true;
  const int *stop = nullptr;  // musg_solver_set_stop_flag

  ~musg_solver() {
    if (exec) cudaGraphExecDestroy(exec);
    if (hst) cudaFreeHost(hst);
  }

  size_t rbytes() const { return precision == MUSG_PRECISION_MIXED ? sizeof(float) : sizeof(double); }

  void create(musg_cell *c, double tol_, unsigned maxiter_, int verbose_, int precision_) {
    require(c != nullptr, MUSG_ERR_ARGUMENT, "null cell");
    require(precision_ == MUSG_PRECISION_FP64 || precision_ == MUSG_PRECISION_MIXED, MUSG_ERR_ARGUMENT,
            "unknown precision");
    cell = c;
    tol = tol_;
    maxiter = maxiter_;
    verbose = verbose_;
    precision = precision_;
    if (precision == MUSG_PRECISION_MIXED) cell->alloc32();
    const size_t n = (size_t)cell->nb_dof();
    x.alloc(n * rbytes());
    r.alloc(n * rbytes());
    p.alloc(n * rbytes());
    // the FP32 inner solve never stores Ap (its last pass updates r directly)
    if (precision != MUSG_PRECISION_MIXED) Ap.alloc(n * rbytes());
    st.alloc(sizeof(CGState));
    MUSG_CUDA(cudaMemset(st.p, 0, sizeof(CGState)));
    MUSG_CUDA(cudaMallocHost(&hst, sizeof(CGState)));
    memset(hst, 0, sizeof(CGState));
    const char *env = getenv("MUSG_CG_GRAPHS");
    if (env && env[0] == '0') graphs = false;
    if (verbose) chunk = 1;
  }

  // one CG iteration (solver_cg.cc:76-97); ev, when given, receives an event
  // before the first and after every kernel (profiling).  FP64: the operator passes
  // (alpha by the last one) and cg_update (x, r, beta); FP32: the operator passes and
  // cg_update_x, which carry the whole iteration (alpha from p.(K:p) in the first pass;
  // r and beta in the last).
  template <typename R> int iteration(cudaStream_t s, cudaEvent_t *ev = nullptr) {
    musg_cell &c = *cell;
    const long long n = c.nb_dof();
    CGState *d = st.as<CGState>();
    double *part = c.partial.as<double>();
    const TangentData<R> td = c.tangent<R>();
    R *ap = sizeof(R) == 8 ? Ap.as<R>() : nullptr;
    const int nop = cg_operator<R>(c.sp, c.tk<R>(), td, d, r.as<R>(), x.as<R>(), p.as<R>(), ap, part, s, ev);
    (void)nop;
    const int k = nb_kernels();
    if (sizeof(R) == 4) return k;
    cg_update<R>(d, x.as<R>(), r.as<R>(), p.as<R>(), Ap.as<R>(), n, part, s);  // and beta
    if (ev) MUSG_CUDA(cudaEventRecord(ev[k], s));
    return k;  // number of kernels
  }

  // kernels per CG iteration: five (3-D) or three (2-D) passes and one vector kernel
  int nb_kernels() const { return cell->dim == 3 ? 6 : 4; }

  static const char *kernel_name(int dim, int precision, int k) {
    static const char *n3[] = {"last_axis_fwd_tangent", "axis1_fwd", "green_axis0", "axis1_inv", "last_axis_inv_dot",
                               "cg_update"};
    static const char *n2[] = {"last_axis_fwd_tangent", "green_axis0", "last_axis_inv_dot", "cg_update"};
    static const char *f3[] = {"last_axis_fwd_tangent_alpha", "cg_update_x", "axis1_fwd", "green_axis0",
                               "axis1_inv", "last_axis_inv_update_r"};
    static const char *f2[] = {"last_axis_fwd_tangent_alpha", "cg_update_x", "green_axis0",
                               "last_axis_inv_update_r"};
    const char *const *t = precision == MUSG_PRECISION_MIXED ? (dim == 3 ? f3 : f2) : (dim == 3 ? n3 : n2);
    const int nk = dim == 3 ? 6 : 4;
    return (k >= 0 && k < nk) ? t[k] : "";
  }

  // mean per-kernel durations (ms) over `iters` eagerly launched iterations started
  // from the cell's last residual, timed with CUDA events on the cell's stream
  template <typename R> int profile(int iters, double *ms) {
    musg_cell &c = *cell;
    cudaStream_t s = c.stream;
    require(c.tangent_valid, MUSG_ERR_RUNTIME, "profile needs an evaluated tangent");
    const long long n = c.nb_dof();
    double *part = c.partial.as<double>();
    cg_init<R>(st.as<CGState>(), c.rhs.as<double>(), r.as<R>(), x.as<R>(), n, 0.0, iters, part, part + 4096, s);
    const int nk = nb_kernels();
    std::vector<cudaEvent_t> ev(nk + 1);
    for (auto &e : ev) MUSG_CUDA(cudaEventCreate(&e));
    std::vector<double> acc(nk, 0.0);
    for (int it = 0; it < iters; ++it) {
      iteration<R>(s, ev.data());
      MUSG_CUDA(cudaEventSynchronize(ev[nk]));
      for (int k = 0; k < nk; ++k) {
        float t = 0;
        MUSG_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
        acc[k] += t;
      }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    for (int k = 0; k < nk; ++k) ms[k] = acc[k] / std::max(iters, 1);
    // leave the solver as after a finished solve (counter untouched by profiling)
    MUSG_CUDA(cudaMemcpyAsync(hst, st.p, sizeof(CGState), cudaMemcpyDeviceToHost, s));
    MUSG_CUDA(cudaStreamSynchronize(s));
    hst->counter = counter;
    MUSG_CUDA(cudaMemcpyAsync(st.p, hst, sizeof(CGState), cudaMemcpyHostToDevice, s));
    MUSG_CUDA(cudaStreamSynchronize(s));
    return nk;
  }

  template <typename R> void build_graph() {
    if (exec) return;
    cudaStream_t s = cell->stream;
    cudaGraph_t g = nullptr;
    const unsigned long long before = g_launches.load();
    MUSG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
    try {
      for (int k = 0; k < chunk; ++k) iteration<R>(s);
    } catch (...) {
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    MUSG_CUDA(cudaStreamEndCapture(s, &g));
    // captured launches did not run; replays account for them
    graph_nodes = g_launches.load() - before;
    g_launches.fetch_sub(graph_nodes);
    MUSG_CUDA(cudaGraphInstantiate(&exec, g, 0));
    cudaGraphDestroy(g);
  }

  // SolverCG::solve (solver_cg.cc:54-110) on a device rhs (FP64 SoA planes)
  template <typename R> void solve_device(const double *rhs) {
    musg_cell &c = *cell;
    cudaStream_t s = c.stream;
    const long long n = c.nb_dof();
    double *part = c.partial.as<double>();
    // r = A 0 - rhs = -rhs, p = -r (first iteration), x = 0
    const double t = (precision == MUSG_PRECISION_MIXED) ? std::max(tol, inner_tol) : tol;
    cg_init<R>(st.as<CGState>(), rhs, r.as<R>(), x.as<R>(), n, t, (int)maxiter, part, part + 4096, s);
    converged = false;
    if (graphs && !verbose) build_graph<R>();
    for (;;) {
      if (exec) {
        MUSG_CUDA(cudaGraphLaunch(exec, s));
        g_launches.fetch_add(graph_nodes);
      } else {
        for (int k = 0; k < chunk; ++k) iteration<R>(s);
      }
      MUSG_CUDA(cudaMemcpyAsync(hst, st.p, sizeof(CGState), cudaMemcpyDeviceToHost, s));
      MUSG_CUDA(cudaStreamSynchronize(s));
      check_stop(stop);
      if (verbose) {
        printf("  at CG step %d: |r|/|b| = %15g, cg_tol = %g\n", hst->iter - 1,
               std::sqrt(hst->rdr / hst->rhs_norm2), tol);
        fflush(stdout);
      }
      if (!hst->active) break;
    }
    if (precision == MUSG_PRECISION_MIXED) {
      unsigned fault = 0;
      MUSG_CUDA(cudaMemcpyAsync(&fault, wait_fault_word(), sizeof fault, cudaMemcpyDeviceToHost, s));
      MUSG_CUDA(cudaStreamSynchronize(s));
      if (fault) {
        MUSG_CUDA(cudaMemsetAsync(wait_fault_word(), 0, sizeof fault, s));
        throw Error(MUSG_ERR_RUNTIME, "a spectral pass timed out waiting for its tile copy; a copy may still land in shared memory after its block exited, so later results of this CUDA context are suspect: check them or restart the process");
      }
    }
    counter = hst->counter;
    if (hst->rdr < hst->tol2) {
      converged = true;
    } else {
      std::ostringstream e;
      e << "Conjugate gradient has not converged. After " << counter << " steps, the solver  FAILED with  |r|/|b| = "
        << std::sqrt(hst->rdr / hst->rhs_norm2) << ", cg_tol = " << std::sqrt(hst->tol2 / hst->rhs_norm2);
      throw Error(MUSG_ERR_CONVERGENCE, e.str());
    }
  }

  void solve_device_any(const double *rhs) {
    if (precision == MUSG_PRECISION_MIXED) solve_device<float>(rhs);
    else solve_device<double>(rhs);
  }

  void reset_counter() {
    counter = 0;
    MUSG_CUDA(cudaMemsetAsync(&st.as<CGState>()->counter, 0, sizeof(unsigned long long), cell->stream));
    MUSG_CUDA(cudaStreamSynchronize(cell->stream));
  }
};

// ---------------------------------------------------------------------- batches
// Same-shape cells solved together: Newton steps in lockstep, every CG iteration one
// launch per pass for all cells (problem b = blockIdx.y), captured in one graph.
struct musg_batch {
  std::vector<musg_cell *> cells;
  std::vector<std::unique_ptr<musg_solver>> solvers;  // per-cell vectors
  int precision = MUSG_PRECISION_FP64;
  double tol = 0, inner_tol = 1e-2;
  unsigned maxiter = 0;
  cudaStream_t stream = nullptr;
  DevBuf states, tab_p, tab_v;
  CGState *hst = nullptr;
  cudaGraphExec_t exec = nullptr;
  unsigned long long graph_nodes = 0;
  int chunk = 16;
  // cells of different grids (the same dimension, formulation and tangent kind): one
  // grouped launch per pass over all of them (generic pass kernels)
  bool uniform = true;
  GroupedOp *gop = nullptr;
  long long nmax = 0;  // the largest cell's vector length
  const int *stop = nullptr;  // musg_batch_set_stop_flag

  ~musg_batch() {
    if (gop) grouped_op_destroy(gop);
    if (exec) cudaGraphExecDestroy(exec);
    if (hst) cudaFreeHost(hst);
    if (stream) cudaStreamDestroy(stream);
  }
  int B() const { return (int)cells.size(); }
  CGState *state(int b) const { return states.as<CGState>() + b; }

  template <typename R> void build_tables() {
    std::vector<ProblemPtrsHost> tp(B());
    std::vector<BatchVec<R>> tv(B());
    for (int b = 0; b < B(); ++b) {
      musg_cell &c = *cells[b];
      musg_solver &sv = *solvers[b];
      const TangentData<R> td = c.tangent<R>();
      tp[b].spec = sizeof(R) == 8 ? c.sp.spec64 : c.sp.spec32;
      tp[b].st = state(b);
      tp[b].r = sv.r.p;
      tp[b].x = sv.x.p;
      tp[b].p = sv.p.p;
      tp[b].Ap = sizeof(R) == 8 ? sv.Ap.p : nullptr;  // the FP32 passes do not store Ap
      tp[b].partial = c.partial.as<double>();
      static_assert(sizeof(TangentData<R>) == sizeof(tp[b].td), "tangent table layout");
      memcpy(tp[b].td, &td, sizeof(td));
      tv[b].st = state(b);
      tv[b].x = sv.x.as<R>();
      tv[b].r = sv.r.as<R>();
      tv[b].p = sv.p.as<R>();
      tv[b].Ap = sv.Ap.as<R>();
      tv[b].partial = c.partial.as<double>();
      tv[b].n = c.nb_dof();
      tv[b].nparts = 0;
      nmax = std::max(nmax, c.nb_dof());
    }
    if (!uniform) {
      std::vector<GroupProblem> probs(B());
      for (int b = 0; b < B(); ++b) {
        probs[b].sp = &cells[b]->sp;
        probs[b].st = state(b);
        probs[b].r = tp[b].r;
        probs[b].x = tp[b].x;
        probs[b].p = tp[b].p;
        probs[b].Ap = tp[b].Ap;
        probs[b].partial = tp[b].partial;
        memcpy(probs[b].td, tp[b].td, sizeof(probs[b].td));
      }
      gop = grouped_op_create<R>(probs, cells[0]->tk<R>());
      for (int b = 0; b < B(); ++b) tv[b].nparts = grouped_op_fwd_partials(gop, b);
    }
    tab_p.alloc(tp.size() * sizeof(ProblemPtrsHost));
    tab_v.alloc(tv.size() * sizeof(BatchVec<R>));
    MUSG_CUDA(cudaMemcpy(tab_p.p, tp.data(), tab_p.bytes, cudaMemcpyHostToDevice));
    MUSG_CUDA(cudaMemcpy(tab_v.p, tv.data(), tab_v.bytes, cudaMemcpyHostToDevice));
  }

  template <typename R> void iteration(cudaStream_t s) {
    musg_cell &c0 = *cells[0];
    if (uniform)
      cg_operator_batch<R>(c0.sp, c0.tk<R>(), (const ProblemPtrs<R> *)tab_p.p, tab_v.as<BatchVec<R>>(), B(),
                           s);  // and alpha (FP32: the whole iteration)
    else
      grouped_op_run<R>(gop, tab_v.as<BatchVec<R>>(), nmax, B(), s);
    if (sizeof(R) == 8) cg_update_batch<R>(tab_v.as<BatchVec<R>>(), nmax, B(), s);  // and beta
  }

  template <typename R> void build_graph() {
    if (exec) return;
    cudaGraph_t g = nullptr;
    const unsigned long long before = g_launches.load();
    MUSG_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeRelaxed));
    try {
      for (int k = 0; k < chunk; ++k) iteration<R>(stream);
    } catch (...) {
      cudaStreamEndCapture(stream, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    MUSG_CUDA(cudaStreamEndCapture(stream, &g));
    graph_nodes = g_launches.load() - before;
    g_launches.fetch_sub(graph_nodes);
    MUSG_CUDA(cudaGraphInstantiate(&exec, g, 0));
    cudaGraphDestroy(g);
  }

  // one batched SolverCG::solve over the cells whose `solve` flag is set
  template <typename R> void solve(const std::vector<char> &solve_it, std::vector<std::string> &errors) {
    const double t = (precision == MUSG_PRECISION_MIXED) ? std::max(tol, inner_tol) : tol;
    for (int b = 0; b < B(); ++b) {
      musg_cell &c = *cells[b];
      double *part = c.partial.as<double>();
      if (solve_it[b]) {
        cg_init<R>(state(b), c.rhs.as<double>(), solvers[b]->r.as<R>(), solvers[b]->x.as<R>(), c.nb_dof(), t,
                   (int)maxiter, part, part + 4096, stream);
      } else {
        MUSG_CUDA(cudaMemsetAsync(&state(b)->active, 0, sizeof(int), stream));
      }
    }
    build_graph<R>();
    for (;;) {
      MUSG_CUDA(cudaGraphLaunch(exec, stream));
      g_launches.fetch_add(graph_nodes);
      MUSG_CUDA(cudaMemcpyAsync(hst, states.p, B() * sizeof(CGState), cudaMemcpyDeviceToHost, stream));
      MUSG_CUDA(cudaStreamSynchronize(stream));
      check_stop(stop);
      bool any = false;
      for (int b = 0; b < B(); ++b) any = any || hst[b].active;
      if (!any) break;
    }
    for (int b = 0; b < B(); ++b) {
      solvers[b]->counter = hst[b].counter;
      if (!solve_it[b]) continue;
      if (!(hst[b].rdr < hst[b].tol2)) {
        std::ostringstream e;
        e << "Conjugate gradient has not converged. After " << hst[b].counter
          << " steps, the solver  FAILED with  |r|/|b| = " << std::sqrt(hst[b].rdr / hst[b].rhs_norm2)
          << ", cg_tol = " << std::sqrt(hst[b].tol2 / hst[b].rhs_norm2);
        errors[b] = e.str();
      }
    }
  }
};

// ---------------------------------------------------------------------- FFT / projection handles
struct musg_fft {
  Spectral sp;
  cudaStream_t stream = nullptr;
  DevBuf a, b;
  ~musg_fft() {
    sp.release();
    if (stream) cudaStreamDestroy(stream);
  }
};

struct musg_projection {
  Spectral sp;
  int kind = 0;
  cudaStream_t stream = nullptr;
  DevBuf a, b;
  ~musg_projection() {
    sp.release();
    if (stream) cudaStreamDestroy(stream);
  }
};

// ---------------------------------------------------------------------- newton_cg
namespace {

constexpr unsigned kLineSearchNewtonMax = 100;

void check_symmetry_or_throw(const double *m, int dim) {
  // solver_common.cc:39-43 with rel_tol = 1e-8
  double n = 0, a = 0;
  for (int j = 0; j < dim; ++j)
    for (int i = 0; i < dim; ++i) {
      n += m[i + dim * j] * m[i + dim * j];
      const double d = m[i + dim * j] - m[j + dim * i];
      a += d * d;
    }
  n = std::sqrt(n);
  a = std::sqrt(a);
  const double rel = 1e-8;
  if (!(rel >= a / n || rel >= n)) throw Error(MUSG_ERR_SOLVER, "all Δε must be symmetric!");
}

// newton_cg (solvers.cc:44-217), or with geus the de Geus variant (solvers.cc:220-408):
// per load step its first Newton iteration solves K dF = -G(K:DF) at the previous
// equilibrium and then applies DF + dF (DF: the macroscopic increment as a field)
void newton_cg_impl(musg_cell *cell, const double *steps, int nsteps, musg_solver *solver, double newton_tol,
                    double equil_tol, int verbose, musg_result_info *infos, double *grads, double *stresses,
                    bool geus = false) {
  require(cell && solver && steps && nsteps > 0, MUSG_ERR_ARGUMENT, "invalid newton_cg arguments");
  require(solver->cell == cell, MUSG_ERR_ARGUMENT, "solver belongs to another cell");
  musg_cell &c = *cell;
  const int dim = c.dim, D2 = c.D2;
  cudaStream_t s = c.stream;
  if (!c.initialised) c.initialise();
  // solvers.cc:98-131: uniform initial strain, load-step checks
  std::vector<double> I(D2, 0.0);
  if (c.form == MUSG_FINITE_STRAIN)
    for (int i = 0; i < dim; ++i) I[i + dim * i] = 1.0;
  else
    for (int k = 0; k < nsteps; ++k) check_symmetry_or_throw(steps + (size_t)k * D2, dim);
  fill_uniform(c.F.as<double>(), c.put_matrix(I.data(), 0), D2, c.npx, s);
  if (verbose > 0) {
    printf("%s for %s strain with\nnewton_tol = %g, cg_tol = %g maxiter = %u\n", geus ? "de Geus-CG" : "Newton-CG",
           c.form == MUSG_FINITE_STRAIN ? "finite" : "small", newton_tol, solver->tol, solver->maxiter);
  }
  std::vector<double> previous(D2, 0.0);
  const long long n = c.nb_dof();
  double *dscal = c.scal.as<double>();
  for (int step = 0; step < nsteps; ++step) {
    const double *macro = steps + (size_t)step * D2;
    std::vector<double> delta(D2);
    for (int k = 0; k < D2; ++k) delta[k] = macro[k] - previous[k];
    double *ddelta = c.put_matrix(delta.data(), 16);
    if (!geus) add_macro(c.F.as<double>(), ddelta, D2, c.npx, s);
    c.residual_kept = false;  // the load step's first residual is projected in FP64
    const bool incremental = solver->precision == MUSG_PRECISION_MIXED && solver->incremental_residual;
    std::string message = "Has not converged";
    double incr_norm = 2 * newton_tol, grad_norm = 1, stress_norm = 2 * equil_tol;
    bool has_converged = false;
    auto convergence_test = [&]() {
      const bool incr_test = incr_norm / grad_norm <= newton_tol;
      const bool stress_test = stress_norm < equil_tol;
      if (incr_test) message = "Residual  tolerance reached";
      else if (stress_test) message = "Reached stress divergence tolerance";
      has_converged = incr_test || stress_test;
      return has_converged;
    };
    unsigned newt_iter = 0;
    bool evaluated = false;  // a line-search trial left P and rhs at the current F
    // the reference bounds the Newton loop by the CG solver's maxiter
    // (solvers.cc:150); with the line search, whose damped steps can creep, at most
    // kLineSearchNewtonMax iterations per load step
    const unsigned newton_max = solver->line_search ? std::min(solver->maxiter, kLineSearchNewtonMax) : solver->maxiter;
    for (; newt_iter < newton_max && !has_converged; ++newt_iter) {
      check_stop(solver->stop);
      const bool first_geus = geus && newt_iter == 0;
      if (evaluated) {
        evaluated = false;
      } else {
        c.evaluate(false);
        if (first_geus) {
          // rhs = -G(K:DF) with DF the uniform macroscopic increment (FP64)
          fill_uniform(c.rhs.as<double>(), ddelta, D2, c.npx, s);
          tangent_operator<double>(c.sp, c.tkind, c.tangent<double>(), c.rhs.as<double>(), c.rhs.as<double>(), s);
          convert<double, double>(c.rhs.as<double>(), c.rhs.as<double>(), n, -1.0, s);
          c.residual_kept = false;
        } else {
          // rhs = -P, projected
          c.project_residual(incremental);
        }
        dot_device<double, double>(c.rhs.as<double>(), c.rhs.as<double>(), n, c.partial.as<double>(), dscal + 32, s);
        MUSG_CUDA(cudaMemcpyAsync(c.hscal + 32, dscal + 32, sizeof(double), cudaMemcpyDeviceToHost, s));
        MUSG_CUDA(cudaStreamSynchronize(s));
        stress_norm = std::sqrt(c.hscal[32]);
      }
      if (convergence_test()) break;
      solver->solve_device_any(c.rhs.as<double>());
      if (first_geus) add_macro(c.F.as<double>(), ddelta, D2, c.npx, s);
      if (solver->line_search && !first_geus) {
        // F = F0 + lam dF for lam = 1, 1/2, ... until the projected residual norm drops
        // below (1 - 1e-4 lam) of the current one (Armijo), or lam = 1/1024; the
        // accepted trial's evaluation serves the next Newton iteration
        if (c.F0.bytes < c.field_bytes()) c.F0.alloc(c.field_bytes());
        MUSG_CUDA(cudaMemcpyAsync(c.F0.p, c.F.p, c.field_bytes(), cudaMemcpyDeviceToDevice, s));
        const double nr = stress_norm;
        for (double lam = 1.0;; lam *= 0.5) {
          if (solver->precision == MUSG_PRECISION_MIXED)
            newton_trial<float>(c.F.as<double>(), c.F0.as<double>(), solver->x.as<float>(), lam, n,
                                c.partial.as<double>(), dscal + 34, s);
          else
            newton_trial<double>(c.F.as<double>(), c.F0.as<double>(), solver->x.as<double>(), lam, n,
                                 c.partial.as<double>(), dscal + 34, s);
          c.evaluate(false);
          c.project_residual(incremental);
          dot_device<double, double>(c.rhs.as<double>(), c.rhs.as<double>(), n, c.partial.as<double>(), dscal + 32, s);
          MUSG_CUDA(cudaMemcpyAsync(c.hscal + 32, dscal + 32, 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
          MUSG_CUDA(cudaStreamSynchronize(s));
          stress_norm = std::sqrt(c.hscal[32]);
          if (stress_norm < (1.0 - 1e-4 * lam) * nr || lam <= 1.0 / 1024) break;
        }
        evaluated = true;
      } else if (solver->precision == MUSG_PRECISION_MIXED) {
        newton_update<float>(c.F.as<double>(), solver->x.as<float>(), n, c.partial.as<double>(), dscal + 34, s);
      } else {
        newton_update<double>(c.F.as<double>(), solver->x.as<double>(), n, c.partial.as<double>(), dscal + 34, s);
      }
      MUSG_CUDA(cudaMemcpyAsync(c.hscal + 34, dscal + 34, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
      MUSG_CUDA(cudaStreamSynchronize(s));
      incr_norm = std::sqrt(c.hscal[34]);
      grad_norm = std::sqrt(c.hscal[35]);
      if (verbose > 0) {
        printf("at Newton step %u, |δ%s|/|Δ%s| = %17g, tol = %g\n", newt_iter, c.form == MUSG_FINITE_STRAIN ? "F" : "ε",
               c.form == MUSG_FINITE_STRAIN ? "F" : "ε", incr_norm / grad_norm, newton_tol);
        fflush(stdout);
      }
      convergence_test();
    }
    previous.assign(macro, macro + D2);
    // mixed precision: the stress of the last evaluation carries the FP32 inner
    // tolerance, so history-free cells return P at the final strain instead
    if (solver->precision == MUSG_PRECISION_MIXED && !c.has_hep) c.evaluate(false);
    const bool conv = convergence_test();
    if (infos) {
      musg_result_info &ri = infos[step];
      ri.success = conv ? 1 : 0;
      ri.status = conv ? 1 : 0;
      ri.nb_it = newt_iter;
      ri.nb_fev = (unsigned)solver->counter;
      memset(ri.message, 0, sizeof(ri.message));
      strncpy(ri.message, message.c_str(), sizeof(ri.message) - 1);
      c.homogenised(ri.hom_stress);
    }
    if (grads) c.download_field(c.F.as<double>(), grads + (size_t)step * n);
    if (stresses) c.download_field(c.P.as<double>(), stresses + (size_t)step * n);
    c.save_history();
  }
  MUSG_CUDA(cudaStreamSynchronize(s));
}

// newton_cg (solvers.cc:44-217) for a batch of cells in lockstep; a cell that fails
// (ConvergenceError) is reported in its result records and leaves the batch
void batch_newton_impl(musg_batch *batch, const double *steps, int nsteps, double newton_tol, double equil_tol,
                       musg_result_info *infos, double *stresses) {
  require(batch && steps && nsteps > 0, MUSG_ERR_ARGUMENT, "invalid batch newton_cg arguments");
  musg_batch &bt = *batch;
  const int B = bt.B();
  musg_cell &c0 = *bt.cells[0];
  const int dim = c0.dim, D2 = c0.D2;
  cudaStream_t s = bt.stream;
  std::vector<cudaStream_t> saved(B);
  for (int b = 0; b < B; ++b) {
    saved[b] = bt.cells[b]->stream;
    bt.cells[b]->stream = s;
  }
  struct Restore {
    musg_batch &bt;
    std::vector<cudaStream_t> &saved;
    ~Restore() {
      for (int b = 0; b < bt.B(); ++b) bt.cells[b]->stream = saved[b];
    }
  } restore{bt, saved};
  std::vector<double> I(D2, 0.0);
  if (c0.form == MUSG_FINITE_STRAIN)
    for (int i = 0; i < dim; ++i) I[i + dim * i] = 1.0;
  else
    for (int k = 0; k < B * nsteps; ++k) check_symmetry_or_throw(steps + (size_t)k * D2, dim);
  for (int b = 0; b < B; ++b)
    fill_uniform(bt.cells[b]->F.as<double>(), bt.cells[b]->put_matrix(I.data(), 0), D2, bt.cells[b]->npx, s);
  std::vector<std::vector<double>> previous(B, std::vector<double>(D2, 0.0));
  std::vector<char> failed(B, 0);
  std::vector<std::string> errmsg(B);
  for (int step = 0; step < nsteps; ++step) {
    std::vector<double> incr(B, 2 * newton_tol), grad(B, 1.0), stress(B, 2 * equil_tol);
    std::vector<char> conv(B, 0), running(B, 0);
    std::vector<unsigned> newt(B, 0);
    std::vector<std::string> message(B, "Has not converged");
    auto test = [&](int b) {
      const bool incr_test = incr[b] / grad[b] <= newton_tol;
      const bool stress_test = stress[b] < equil_tol;
      if (incr_test) message[b] = "Residual  tolerance reached";
      else if (stress_test) message[b] = "Reached stress divergence tolerance";
      conv[b] = incr_test || stress_test;
      return (bool)conv[b];
    };
    for (int b = 0; b < B; ++b) {
      if (failed[b]) continue;
      musg_cell &c = *bt.cells[b];
      const double *macro = steps + ((size_t)b * nsteps + step) * D2;
      std::vector<double> delta(D2);
      for (int k = 0; k < D2; ++k) delta[k] = macro[k] - previous[b][k];
      add_macro(c.F.as<double>(), c.put_matrix(delta.data(), 16), D2, c.npx, s);
      previous[b].assign(macro, macro + D2);
      running[b] = 1;
      c.residual_kept = false;
    }
    for (;;) {
      check_stop(bt.stop);
      // Newton iteration: evaluate, residual, convergence (per cell)
      std::vector<char> solve_it(B, 0);
      bool any = false;
      for (int b = 0; b < B; ++b) {
        if (!running[b] || newt[b] >= bt.maxiter) {
          running[b] = 0;
          continue;
        }
        musg_cell &c = *bt.cells[b];
        c.evaluate(false);
        c.project_residual(bt.precision == MUSG_PRECISION_MIXED && bt.solvers[b]->incremental_residual);
        dot_device<double, double>(c.rhs.as<double>(), c.rhs.as<double>(), c.nb_dof(), c.partial.as<double>(),
                                   c.scal.as<double>() + 32, s);
        MUSG_CUDA(cudaMemcpyAsync(c.hscal + 32, c.scal.as<double>() + 32, sizeof(double), cudaMemcpyDeviceToHost, s));
      }
      MUSG_CUDA(cudaStreamSynchronize(s));
      for (int b = 0; b < B; ++b) {
        if (!running[b]) continue;
        stress[b] = std::sqrt(bt.cells[b]->hscal[32]);
        if (test(b)) {
          running[b] = 0;
          continue;
        }
        solve_it[b] = 1;
        any = true;
      }
      if (!any) break;
      std::vector<std::string> errors(B);
      if (bt.precision == MUSG_PRECISION_MIXED) bt.solve<float>(solve_it, errors);
      else bt.solve<double>(solve_it, errors);
      for (int b = 0; b < B; ++b) {
        if (!solve_it[b]) continue;
        if (!errors[b].empty()) {
          failed[b] = 1;
          running[b] = 0;
          errmsg[b] = errors[b];
          continue;
        }
        musg_cell &c = *bt.cells[b];
        double *dscal = c.scal.as<double>();
        if (bt.precision == MUSG_PRECISION_MIXED)
          newton_update<float>(c.F.as<double>(), bt.solvers[b]->x.as<float>(), c.nb_dof(), c.partial.as<double>(),
                               dscal + 34, s);
        else
          newton_update<double>(c.F.as<double>(), bt.solvers[b]->x.as<double>(), c.nb_dof(), c.partial.as<double>(),
                                dscal + 34,
                                s);
        MUSG_CUDA(cudaMemcpyAsync(c.hscal + 34, dscal + 34, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
      }
      MUSG_CUDA(cudaStreamSynchronize(s));
      for (int b = 0; b < B; ++b) {
        if (!solve_it[b] || failed[b]) continue;
        incr[b] = std::sqrt(bt.cells[b]->hscal[34]);
        grad[b] = std::sqrt(bt.cells[b]->hscal[35]);
        test(b);
        newt[b] += 1;
        if (conv[b]) running[b] = 0;
      }
    }
    for (int b = 0; b < B; ++b) {
      musg_cell &c = *bt.cells[b];
      if (!failed[b] && bt.precision == MUSG_PRECISION_MIXED && !c.has_hep) c.evaluate(false);
      musg_result_info &ri = infos[(size_t)b * nsteps + step];
      const bool ok = !failed[b] && test(b);
      ri.success = ok ? 1 : 0;
      ri.status = ok ? 1 : 0;
      ri.nb_it = newt[b];
      ri.nb_fev = (unsigned)bt.solvers[b]->counter;
      memset(ri.message, 0, sizeof(ri.message));
      strncpy(ri.message, failed[b] ? errmsg[b].c_str() : message[b].c_str(), sizeof(ri.message) - 1);
      if (!failed[b]) c.homogenised(ri.hom_stress);
      else std::fill(ri.hom_stress, ri.hom_stress + 9, std::nan(""));
      if (stresses && !failed[b]) {
        // cells one after another, each nb_steps x its nb_dof (the uniform layout when all match)
        size_t off = 0;
        for (int k = 0; k < b; ++k) off += (size_t)nsteps * bt.cells[k]->nb_dof();
        c.download_field(c.P.as<double>(), stresses + off + (size_t)step * c.nb_dof());
      }
      if (!failed[b]) c.save_history();
    }
  }
  MUSG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

// ====================================================================== C ABI
namespace {
template <typename R> void cg_operator_once(musg_cell &c, const double *dF, double *dP) {
  const long long n = c.nb_dof();
  if (c.io2.bytes < c.field_bytes()) c.io2.alloc(c.field_bytes());
  c.upload_field(dF, c.io2.as<double>());
  DevBuf r, x, p, Ap, st;
  r.alloc((size_t)n * sizeof(R));
  x.alloc((size_t)n * sizeof(R));
  p.alloc((size_t)n * sizeof(R));
  Ap.alloc((size_t)n * sizeof(R));
  MUSG_CUDA(cudaMemsetAsync(x.p, 0, (size_t)n * sizeof(R), c.stream));
  st.alloc(sizeof(CGState));
  // first CG iteration: p = -r, so r = -dF gives p = dF and Ap = G(K:dF)
  convert<R, double>(r.as<R>(), c.io2.as<double>(), n, -1.0, c.stream);
  CGState h{};
  h.maxiter = 1;
  h.active = 1;
  MUSG_CUDA(cudaMemcpyAsync(st.p, &h, sizeof(h), cudaMemcpyHostToDevice, c.stream));
  // the kernels of the solver's iteration; the FP32 ones store Ap because it is given
  cg_operator<R>(c.sp, c.tk<R>(), c.tangent<R>(), st.as<CGState>(), r.as<R>(), x.as<R>(), p.as<R>(), Ap.as<R>(),
                 c.partial.as<double>(), c.stream);
  convert<double, R>(c.io2.as<double>(), Ap.as<R>(), n, 1.0, c.stream);
  c.download_field(c.io2.as<double>(), dP);
}
}  // namespace

extern "C" {

const char *musg_last_error(void) { return g_last_error.c_str(); }

int musg_version(void) { return 100; }

int musg_selftest_wait_timeout(double limit_ms, int *timed_out) {
  return guard([&] {
    require(timed_out && limit_ms > 0 && limit_ms < 10000, MUSG_ERR_ARGUMENT, "limit_ms in (0, 10000) and an output");
    cudaStream_t s = nullptr;
    MUSG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    unsigned fault = 0;
    try {
      MUSG_CUDA(cudaMemsetAsync(wait_fault_word(), 0, sizeof fault, s));
      wait_probe((unsigned long long)(limit_ms * 1e6), s);
      MUSG_CUDA(cudaMemcpyAsync(&fault, wait_fault_word(), sizeof fault, cudaMemcpyDeviceToHost, s));
      MUSG_CUDA(cudaMemsetAsync(wait_fault_word(), 0, sizeof fault, s));
      MUSG_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
      cudaStreamDestroy(s);
      throw;
    }
    cudaStreamDestroy(s);
    *timed_out = fault ? 1 : 0;
  });
}

int musg_set_device(int device) {
  return guard([&] { MUSG_CUDA(cudaSetDevice(device)); });
}

int musg_device_count(int *count) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  if (count) *count = n;
  return MUSG_OK;
}

int musg_cell_create(int dim, const int *resolutions, const double *lengths, int formulation, int flags,
                     musg_cell **out) {
  return guard([&] {
    require(out && resolutions, MUSG_ERR_ARGUMENT, "null argument");
    auto c = std::make_unique<musg_cell>();
    c->create(dim, resolutions, lengths, formulation, flags);
    *out = c.release();
  });
}

int musg_cell_destroy(musg_cell *cell) {
  return guard([&] { delete cell; });
}

int musg_cell_sizes(musg_cell *cell, long long *nb_dof, long long *nb_pixels) {
  return guard([&] {
    require(cell, MUSG_ERR_ARGUMENT, "null cell");
    if (nb_dof) *nb_dof = cell->nb_dof();
    if (nb_pixels) *nb_pixels = cell->npx;
  });
}

int musg_cell_set_stream(musg_cell *cell, void *cuda_stream) {
  return guard([&] {
    require(cell, MUSG_ERR_ARGUMENT, "null cell");
    MUSG_CUDA(cudaStreamSynchronize(cell->stream));
    if (cell->own_stream) cudaStreamDestroy(cell->stream);
    cell->own_stream = false;
    cell->stream = (cudaStream_t)cuda_stream;
  });
}

int musg_material_create(musg_cell *cell, int law, const char *name, const double *params, int nb_params,
                         int *material) {
  return guard([&] {
    require(cell, MUSG_ERR_ARGUMENT, "null cell");
    require(!cell->initialised, MUSG_ERR_RUNTIME, "cannot add materials to an initialised cell");
    Material m;
    m.law = law;
    m.name = name ? name : "";
    switch (law) {
      case MUSG_LAW_LE1:
      case MUSG_LAW_LE2:
        require(nb_params >= 2, MUSG_ERR_ARGUMENT, "this material needs (Young, Poisson)");
        m.E = params[0];
        m.nu = params[1];
        m.stride = law == MUSG_LAW_LE2 ? cell->D2 : 0;
        break;
      case MUSG_LAW_LE3:
      case MUSG_LAW_LE4:
        m.stride = 2;
        break;
      case MUSG_LAW_GENERIC: {
        const int vs = cell->dim == 2 ? 3 : 6;
        if (nb_params != vs * vs) {
          std::ostringstream err;
          err << "The stiffness tensor should be input as a " << vs << " × " << vs
              << " Matrix in Voigt notation. You supplied " << nb_params << " values";
          throw Error(MUSG_ERR_ARGUMENT, err.str());
        }
        m.C = stiffness_from_voigt(params, cell->dim);
        break;
      }
      case MUSG_LAW_HEP1:
        require(nb_params >= 4, MUSG_ERR_ARGUMENT, "this material needs (Young, Poisson, tau_y0, H)");
        m.E = params[0];
        m.nu = params[1];
        m.tau_y0 = params[2];
        m.H = params[3];
        m.logm_mode = nb_params >= 5 ? (int)params[4] : 0;
        require(m.logm_mode >= 0 && m.logm_mode <= kHep1Consistent, MUSG_ERR_ARGUMENT,
                "HEP1 mode: 0 projector logm, 1 spectral logm, 2 spectral logm with the consistent tangent");
        break;
      default:
        throw Error(MUSG_ERR_ARGUMENT, "unknown material law");
    }
    cell->materials.push_back(std::move(m));
    if (material) *material = (int)cell->materials.size() - 1;
  });
}

int musg_material_add_pixels(musg_cell *cell, int material, const long long *pixels, long long count,
                             const double *per_pixel, int stride) {
  return guard([&] {
    require(cell, MUSG_ERR_ARGUMENT, "null cell");
    require(!cell->initialised, MUSG_ERR_RUNTIME, "cannot add pixels to an initialised cell");
    require(material >= 0 && material < (int)cell->materials.size(), MUSG_ERR_ARGUMENT, "unknown material");
    Material &m = cell->materials[material];
    if (m.stride > 0) {
      if (m.law == MUSG_LAW_LE2)
        require(per_pixel && stride == m.stride, MUSG_ERR_RUNTIME, "this material needs pixels with and eigenstrain");
      else
        require(per_pixel && stride == m.stride, MUSG_ERR_RUNTIME,
                "this material needs pixels with Youngs modulus and Poisson ratio.");
    }
    require(count >= 0 && (count == 0 || pixels), MUSG_ERR_ARGUMENT, "null pixel list");
    bool in_range = true;
    for (long long k = 0; k < count; ++k) in_range &= pixels[k] >= 0 && pixels[k] < cell->npx;
    require(in_range, MUSG_ERR_ARGUMENT, "pixel index out of range");
    m.pixels.insert(m.pixels.end(), pixels, pixels + count);
    if (m.stride > 0) m.per_pixel.insert(m.per_pixel.end(), per_pixel, per_pixel + count * (long long)m.stride);
  });
}

int musg_material_size(musg_cell *cell, int material, long long *count) {
  return guard([&] {
    require(cell && material >= 0 && material < (int)cell->materials.size(), MUSG_ERR_ARGUMENT, "unknown material");
    *count = (long long)cell->materials[material].pixels.size();
  });
}

int musg_cell_initialise(musg_cell *cell, int plan_flags) {
  return guard([&] {
    require(cell, MUSG_ERR_ARGUMENT, "null cell");
    require(plan_flags >= 0 && plan_flags <= 2, MUSG_ERR_ARGUMENT, "unknown planner flag type");
    cell->plan_flags = plan_flags;
    cell->initialise();
  });
}

int musg_cell_tuning(musg_cell *cell, int *threads, long long *bytes) {
  return guard([&] {
    require(cell && threads && bytes, MUSG_ERR_ARGUMENT, "null argument");
    for (int p = 0; p < 2; ++p)
      for (int k = 0; k < 3; ++k) {
        threads[3 * p + k] = cell->sp.tune_threads[p][k];
        bytes[3 * p + k] = cell->sp.tune_bytes[p][k];
      }
  });
}

int musg_cell_set_uniform_strain(musg_cell *cell, const double *strain) {
  return guard([&] {
    require(cell && strain, MUSG_ERR_ARGUMENT, "null argument");
    fill_uniform(cell->F.as<double>(), cell->put_matrix(strain, 0), cell->D2, cell->npx, cell->stream);
    MUSG_CUDA(cudaStreamSynchronize(cell->stream));
  });
}

int musg_cell_get_strain(musg_cell *cell, double *out) {
  return guard([&] {
    require(cell && out, MUSG_ERR_ARGUMENT, "null argument");
    if (!cell->initialised) cell->initialise();  // CellBase::get_strain initialises
    cell->download_field(cell->F.as<double>(), out);
  });
}

int musg_cell_set_strain(musg_cell *cell, const double *in) {
  return guard([&] {
    require(cell && in, MUSG_ERR_ARGUMENT, "null argument");
    cell->upload_field(in, cell->F.as<double>());
    MUSG_CUDA(cudaStreamSynchronize(cell->stream));
  });
}

int musg_cell_get_stress(musg_cell *cell, double *out) {
  return guard([&] {
    require(cell && out, MUSG_ERR_ARGUMENT, "null argument");
    cell->download_field(cell->P.as<double>(), out);
  });
}

int musg_cell_homogenised_stress(musg_cell *cell, double *out) {
  return guard([&] {
    require(cell && out, MUSG_ERR_ARGUMENT, "null argument");
    musg_cell &c = *cell;
    require(c.initialised, MUSG_ERR_RUNTIME, "the cell is not initialised");
    double *d = c.scal.as<double>() + 40;
    plane_means(c.P.as<double>(), c.D2, c.npx, c.partial.as<double>(), d, c.stream);
    MUSG_CUDA(cudaMemcpyAsync(out, d, c.D2 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    MUSG_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int musg_cell_evaluate_stress_tangent(musg_cell *cell, double *stress_out, double *tangent_out) {
  return guard([&] {
    require(cell, MUSG_ERR_ARGUMENT, "null cell");
    cell->evaluate(tangent_out != nullptr);
    if (stress_out) cell->download_field(cell->P.as<double>(), stress_out);
    if (tangent_out) {
      const size_t bytes = (size_t)cell->nb_dof() * cell->D2 * sizeof(double);
      MUSG_CUDA(cudaMemcpyAsync(tangent_out, cell->Kfull.p, bytes, cudaMemcpyDeviceToHost, cell->stream));
    }
    MUSG_CUDA(cudaStreamSynchronize(cell->stream));
  });
}

int musg_cell_apply_projection(musg_cell *cell, double *vec) {
  return guard([&] {
    require(cell && vec, MUSG_ERR_ARGUMENT, "null argument");
    musg_cell &c = *cell;
    if (c.io2.bytes < c.field_bytes()) c.io2.alloc(c.field_bytes());
    c.upload_field(vec, c.io2.as<double>());
    spectral_project<double>(c.sp, c.io2.as<double>(), c.io2.as<double>(), 1.0, c.stream);
    c.download_field(c.io2.as<double>(), vec);
  });
}

int musg_cell_directional_stiffness(musg_cell *cell, const double *dF, double *dP) {
  return guard([&] {
    require(cell && dF && dP, MUSG_ERR_ARGUMENT, "null argument");
    musg_cell &c = *cell;
    require(c.tangent_valid, MUSG_ERR_RUNTIME,
            "currently only implemented for cases where a stiffness matrix exists");
    if (c.io2.bytes < c.field_bytes()) c.io2.alloc(c.field_bytes());
    c.upload_field(dF, c.io2.as<double>());
    tangent_operator<double>(c.sp, c.tkind, c.tangent<double>(), c.io2.as<double>(), c.io2.as<double>(), c.stream);
    c.download_field(c.io2.as<double>(), dP);
  });
}

int musg_cell_cg_operator(musg_cell *cell, int precision, const double *dF, double *dP) {
  return guard([&] {
    require(cell && dF && dP, MUSG_ERR_ARGUMENT, "null argument");
    require(precision == MUSG_PRECISION_FP64 || precision == MUSG_PRECISION_MIXED, MUSG_ERR_ARGUMENT,
            "unknown precision");
    musg_cell &c = *cell;
    require(c.tangent_valid, MUSG_ERR_RUNTIME,
            "currently only implemented for cases where a stiffness matrix exists");
    if (precision == MUSG_PRECISION_FP64) {
      cg_operator_once<double>(c, dF, dP);
      return;
    }
    if (!c.need32 || !c.lam32.p) {
      c.alloc32();
      c.evaluate(false);  // the FP32 tangent data of the current strain
    }
    cg_operator_once<float>(c, dF, dP);
  });
}

int musg_cell_save_history_variables(musg_cell *cell) {
  return guard([&] {
    require(cell, MUSG_ERR_ARGUMENT, "null cell");
    cell->save_history();
  });
}

int musg_cell_get_internal(musg_cell *cell, const char *name, double *out, long long capacity, int *nb_components) {
  return guard([&] {
    require(cell && name, MUSG_ERR_ARGUMENT, "null argument");
    musg_cell &c = *cell;
    const int D = c.dim, D2 = c.D2;
    // the internal fields of the reference's materials and where their values live
    enum Src { EIG, CT4, LAM, MU, EPS, FPREV, BE };
    struct Spec {
      int law, ncomp, src, slot;
    } sp{0, 0, 0, 0};
    const std::string n = name;
    const std::string sub = ", sub_field index ";
    // HEP1 state fields (material_hyper_elasto_plastic1.cc:46-53), two sub-fields
    // each (statefield.hh:181-188)
    const char *hep_prefix[3] = {"cumulated plastic flow \xce\xb5\xe2\x82\x9a",
                                 "Previous placement gradient F\xe1\xb5\x97",
                                 "Previous left Cauchy-Green deformation b\xe2\x82\x91\xe1\xb5\x97"};
    bool found = false;
    if (n == "Eigenstrain") sp = {MUSG_LAW_LE2, D2, EIG, 0}, found = true;             // material_linear_elastic2.cc:44
    else if (n == "local stiffness tensor") sp = {MUSG_LAW_LE3, D2 * D2, CT4, 0}, found = true;  // ..._elastic3.cc:45
    else if (n == "local first Lame constant") sp = {MUSG_LAW_LE4, 1, LAM, 0}, found = true;    // ..._elastic4.cc:47
    else if (n == "local second Lame constant(shear modulus)") sp = {MUSG_LAW_LE4, 1, MU, 0}, found = true;
    for (int k = 0; k < 3 && !found; ++k)
      for (int slot = 0; slot < 2 && !found; ++slot)
        if (n == std::string(hep_prefix[k]) + sub + std::to_string(slot)) {
          sp = {MUSG_LAW_HEP1, k == 0 ? 1 : D2, k == 0 ? EPS : k == 1 ? FPREV : BE, slot};
          found = true;
        }
    bool owned = false;
    for (const Material &mt : c.materials) owned = owned || (found && mt.law == sp.law);
    require(owned, MUSG_ERR_RUNTIME,
            "The field named '" + n + "' does not exist in any of the materials and can therefore not be globalised!");
    if (nb_components) *nb_components = sp.ncomp;
    if (!out) return;
    require(capacity >= (long long)sp.ncomp * c.npx, MUSG_ERR_SHAPE, "output array too small");
    if (!c.initialised) c.initialise();
    // the device planes behind the field
    std::vector<const double *> planes;
    auto field = [&](const DevBuf &b, int nplanes) {
      for (int k = 0; k < nplanes; ++k) planes.push_back(b.as<double>() + (size_t)k * c.npx);
    };
    switch (sp.src) {
      case EIG: field(c.eig, D2); break;
      case CT4:
      case LAM: field(c.lam64, 1); if (sp.src == CT4) field(c.mu64, 1); break;
      case MU: field(c.mu64, 1); break;
      case EPS: field(c.eps[sp.slot], 1); break;
      case FPREV: field(c.Fprev[sp.slot], D2); break;
      default: field(c.be[sp.slot], D2); break;
    }
    std::vector<double> h(planes.size() * (size_t)c.npx);
    MUSG_CUDA(cudaStreamSynchronize(c.stream));
    for (size_t k = 0; k < planes.size(); ++k)
      MUSG_CUDA(cudaMemcpy(h.data() + k * c.npx, planes[k], c.plane_bytes(), cudaMemcpyDeviceToHost));
    std::fill(out, out + (size_t)sp.ncomp * c.npx, 0.0);
    for (const Material &mt : c.materials) {
      if (mt.law != sp.law) continue;
      for (long long p : mt.pixels) {
        double *o = out + (size_t)p * sp.ncomp;
        if (sp.src == CT4) {
          // C = lam I (x) I + 2 mu I_sym (materials_toolbox.hh:638-652), T4 layout
          const double lam = h[p], mu = h[c.npx + p];
          for (int l = 0; l < D; ++l)
            for (int k = 0; k < D; ++k)
              for (int j = 0; j < D; ++j)
                for (int i = 0; i < D; ++i)
                  o[(i + D * j) + D2 * (k + D * l)] =
                      (i == j && k == l ? lam : 0.0) + mu * ((i == k && j == l ? 1.0 : 0.0) + (i == l && j == k ? 1.0 : 0.0));
        } else {
          for (int q = 0; q < sp.ncomp; ++q) o[q] = h[(size_t)q * c.npx + p];
        }
      }
    }
  });
}

namespace {
// checkpoint image: header, then the strain and stress fields and (HEP1) the six
// state planes sets, all as stored on the device (component planes)
struct CheckpointHeader {
  char magic[8];
  int dim, res[3], form, has_hep, hep_cur, nbufs;
  long long npx;
};
std::vector<std::pair<DevBuf *, size_t>> checkpoint_buffers(musg_cell &c) {
  std::vector<std::pair<DevBuf *, size_t>> b{{&c.F, c.field_bytes()}, {&c.P, c.field_bytes()}};
  if (c.has_hep)
    for (int k = 0; k < 2; ++k) {
      b.push_back({&c.Fprev[k], c.field_bytes()});
      b.push_back({&c.be[k], c.field_bytes()});
      b.push_back({&c.eps[k], c.plane_bytes()});
    }
  return b;
}
}  // namespace

int musg_cell_checkpoint_size(musg_cell *cell, unsigned long long *bytes) {
  return guard([&] {
    require(cell && bytes, MUSG_ERR_ARGUMENT, "null argument");
    if (!cell->initialised) cell->initialise();
    unsigned long long b = sizeof(CheckpointHeader);
    for (auto &e : checkpoint_buffers(*cell)) b += e.second;
    *bytes = b;
  });
}

int musg_cell_checkpoint_save(musg_cell *cell, void *buf, unsigned long long bytes) {
  return guard([&] {
    require(cell && buf, MUSG_ERR_ARGUMENT, "null argument");
    musg_cell &c = *cell;
    if (!c.initialised) c.initialise();
    auto bufs = checkpoint_buffers(c);
    unsigned long long need = sizeof(CheckpointHeader);
    for (auto &e : bufs) need += e.second;
    require(bytes >= need, MUSG_ERR_SHAPE, "checkpoint buffer too small");
    CheckpointHeader h{};
    memcpy(h.magic, "MUSGCKP1", 8);
    h.dim = c.dim;
    for (int d = 0; d < 3; ++d) h.res[d] = c.res[d];
    h.form = c.form;
    h.has_hep = c.has_hep;
    h.hep_cur = c.hep_cur;
    h.nbufs = (int)bufs.size();
    h.npx = c.npx;
    char *o = (char *)buf;
    memcpy(o, &h, sizeof(h));
    o += sizeof(h);
    MUSG_CUDA(cudaStreamSynchronize(c.stream));
    for (auto &e : bufs) {
      MUSG_CUDA(cudaMemcpy(o, e.first->p, e.second, cudaMemcpyDeviceToHost));
      o += e.second;
    }
  });
}

int musg_cell_checkpoint_load(musg_cell *cell, const void *buf, unsigned long long bytes) {
  return guard([&] {
    require(cell && buf, MUSG_ERR_ARGUMENT, "null argument");
    musg_cell &c = *cell;
    if (!c.initialised) c.initialise();
    require(bytes >= sizeof(CheckpointHeader), MUSG_ERR_SHAPE, "checkpoint too short");
    CheckpointHeader h;
    memcpy(&h, buf, sizeof(h));
    require(memcmp(h.magic, "MUSGCKP1", 8) == 0, MUSG_ERR_ARGUMENT, "not a cell checkpoint");
    auto bufs = checkpoint_buffers(c);
    require(h.dim == c.dim && h.res[0] == c.res[0] && h.res[1] == c.res[1] && h.res[2] == c.res[2] &&
                h.form == c.form && h.has_hep == (int)c.has_hep && h.npx == c.npx && h.nbufs == (int)bufs.size(),
            MUSG_ERR_SHAPE, "the checkpoint belongs to a cell of another shape or material kind");
    unsigned long long need = sizeof(CheckpointHeader);
    for (auto &e : bufs) need += e.second;
    require(bytes >= need, MUSG_ERR_SHAPE, "checkpoint too short");
    const char *i = (const char *)buf + sizeof(h);
    MUSG_CUDA(cudaStreamSynchronize(c.stream));
    for (auto &e : bufs) {
      MUSG_CUDA(cudaMemcpy(e.first->p, i, e.second, cudaMemcpyHostToDevice));
      i += e.second;
    }
    c.hep_cur = h.hep_cur;
    c.tangent_valid = false;  // re-evaluated at the restored strain by the next solve
  });
}

int musg_solver_cg_create(musg_cell *cell, double tol, unsigned maxiter, int verbose, int precision,
                          musg_solver **out) {
  return guard([&] {
    require(out, MUSG_ERR_ARGUMENT, "null argument");
    auto s = std::make_unique<musg_solver>();
    s->create(cell, tol, maxiter, verbose, precision);
    *out = s.release();
  });
}

int musg_solver_set_line_search(musg_solver *solver, int enable) {
  return guard([&] {
    require(solver, MUSG_ERR_ARGUMENT, "null solver");
    solver->line_search = enable != 0;
  });
}

int musg_solver_set_stop_flag(musg_solver *solver, const int *flag) {
  return guard([&] {
    require(solver, MUSG_ERR_ARGUMENT, "null solver");
    solver->stop = flag;
  });
}

int musg_batch_set_stop_flag(musg_batch *batch, const int *flag) {
  return guard([&] {
    require(batch, MUSG_ERR_ARGUMENT, "null batch");
    batch->stop = flag;
  });
}

int musg_solver_set_incremental_residual(musg_solver *solver, int enable) {
  return guard([&] {
    require(solver, MUSG_ERR_ARGUMENT, "null solver");
    solver->incremental_residual = enable != 0;
  });
}

int musg_solver_set_inner_tol(musg_solver *solver, double inner_tol) {
  return guard([&] {
    require(solver && inner_tol >= 0, MUSG_ERR_ARGUMENT, "invalid argument");
    solver->inner_tol = inner_tol;
  });
}

int musg_solver_destroy(musg_solver *solver) {
  return guard([&] { delete solver; });
}

int musg_solver_get_counter(musg_solver *solver, unsigned *counter) {
  return guard([&] {
    require(solver && counter, MUSG_ERR_ARGUMENT, "null argument");
    *counter = (unsigned)solver->counter;
  });
}

int musg_solver_reset_counter(musg_solver *solver) {
  return guard([&] {
    require(solver, MUSG_ERR_ARGUMENT, "null solver");
    solver->reset_counter();
  });
}

int musg_solver_has_converged(musg_solver *solver, int *converged) {
  return guard([&] {
    require(solver && converged, MUSG_ERR_ARGUMENT, "null argument");
    *converged = solver->converged ? 1 : 0;
  });
}

int musg_solver_solve(musg_solver *solver, const double *rhs, double *x_out) {
  return guard([&] {
    require(solver && rhs && x_out, MUSG_ERR_ARGUMENT, "null argument");
    musg_cell &c = *solver->cell;
    require(c.tangent_valid, MUSG_ERR_RUNTIME, "currently only implemented for cases where a stiffness matrix exists");
    if (c.io2.bytes < c.field_bytes()) c.io2.alloc(c.field_bytes());
    c.upload_field(rhs, c.io2.as<double>());
    solver->solve_device_any(c.io2.as<double>());
    if (solver->precision == MUSG_PRECISION_MIXED)
      convert<double, float>(c.io2.as<double>(), solver->x.as<float>(), c.nb_dof(), 1.0, c.stream);
    else
      convert<double, double>(c.io2.as<double>(), solver->x.as<double>(), c.nb_dof(), 1.0, c.stream);
    c.download_field(c.io2.as<double>(), x_out);
  });
}

int musg_probe_fp64_fma(double *tflops) {
  return guard([&] {
    require(tflops, MUSG_ERR_ARGUMENT, "null argument");
    *tflops = fp64_fma_tflops(nullptr);
  });
}

int musg_launch_count(unsigned long long *count) {
  return guard([&] {
    require(count, MUSG_ERR_ARGUMENT, "null argument");
    *count = g_launches.load();
  });
}

int musg_solver_profile(musg_solver *solver, int iterations, double *ms_out, int *nb_kernels) {
  return guard([&] {
    require(solver && ms_out && iterations > 0, MUSG_ERR_ARGUMENT, "invalid argument");
    const int nk = solver->precision == MUSG_PRECISION_MIXED ? solver->profile<float>(iterations, ms_out)
                                                             : solver->profile<double>(iterations, ms_out);
    if (nb_kernels) *nb_kernels = nk;
  });
}

const char *musg_solver_kernel_name(musg_solver *solver, int k) {
  if (!solver || !solver->cell) return "";
  return musg_solver::kernel_name(solver->cell->dim, solver->precision, k);
}

int musg_batch_create(musg_cell **cells, int nb_cells, double tol, unsigned maxiter, int precision,
                      musg_batch **out) {
  return guard([&] {
    require(out && cells && nb_cells > 0, MUSG_ERR_ARGUMENT, "invalid argument");
    auto bt = std::make_unique<musg_batch>();
    musg_cell &c0 = *cells[0];
    for (int b = 0; b < nb_cells; ++b) {
      musg_cell &c = *cells[b];
      require(cells[b] != nullptr, MUSG_ERR_ARGUMENT, "null cell");
      if (!c.initialised) c.initialise();
      require(c.dim == c0.dim && c.form == c0.form && c.flags == c0.flags && c.tkind == c0.tkind &&
                  c.tkind32 == c0.tkind32,
              MUSG_ERR_ARGUMENT, "cells of a batch need the same dimension, formulation and material-law kind");
      if (c.res[0] != c0.res[0] || c.res[1] != c0.res[1] || c.res[2] != c0.res[2]) bt->uniform = false;
      for (int k = 0; k < b; ++k) require(cells[k] != cells[b], MUSG_ERR_ARGUMENT, "a cell appears twice in a batch");
      auto sv = std::make_unique<musg_solver>();
      sv->create(&c, tol, maxiter, 0, precision);
      bt->solvers.push_back(std::move(sv));
      bt->cells.push_back(&c);
    }
    // the launch shapes of the first cell serve the whole batch
    for (int b = 1; b < nb_cells; ++b)
      for (int p = 0; p < 2; ++p)
        for (int k = 0; k < 3; ++k) {
          cells[b]->sp.tune_threads[p][k] = c0.sp.tune_threads[p][k];
          cells[b]->sp.tune_bytes[p][k] = c0.sp.tune_bytes[p][k];
        }
    bt->precision = precision;
    bt->tol = tol;
    bt->maxiter = maxiter;
    MUSG_CUDA(cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking));
    bt->states.alloc(nb_cells * sizeof(CGState));
    MUSG_CUDA(cudaMemset(bt->states.p, 0, bt->states.bytes));
    MUSG_CUDA(cudaMallocHost(&bt->hst, nb_cells * sizeof(CGState)));
    if (precision == MUSG_PRECISION_MIXED) bt->build_tables<float>();
    else bt->build_tables<double>();
    *out = bt.release();
  });
}

int musg_batch_destroy(musg_batch *batch) {
  return guard([&] { delete batch; });
}

int musg_batch_set_inner_tol(musg_batch *batch, double inner_tol) {
  return guard([&] {
    require(batch && inner_tol >= 0, MUSG_ERR_ARGUMENT, "invalid argument");
    batch->inner_tol = inner_tol;
  });
}

int musg_batch_newton_cg(musg_batch *batch, const double *load_steps, int nb_steps, double newton_tol,
                         double equil_tol, musg_result_info *infos, double *stresses) {
  return guard([&] {
    require(infos, MUSG_ERR_ARGUMENT, "null result records");
    batch_newton_impl(batch, load_steps, nb_steps, newton_tol, equil_tol, infos, stresses);
  });
}

int musg_newton_cg(musg_cell *cell, const double *load_steps, int nb_steps, musg_solver *solver, double newton_tol,
                   double equil_tol, int verbose, musg_result_info *infos, double *grads, double *stresses) {
  return guard([&] {
    newton_cg_impl(cell, load_steps, nb_steps, solver, newton_tol, equil_tol, verbose, infos, grads, stresses);
  });
}

int musg_de_geus(musg_cell *cell, const double *load_steps, int nb_steps, musg_solver *solver, double newton_tol,
                 double equil_tol, int verbose, musg_result_info *infos, double *grads, double *stresses) {
  return guard([&] {
    newton_cg_impl(cell, load_steps, nb_steps, solver, newton_tol, equil_tol, verbose, infos, grads, stresses, true);
  });
}

int musg_fft_create(int dim, const int *resolutions, int nb_components, musg_fft **out) {
  return guard([&] {
    require(out && resolutions && nb_components > 0, MUSG_ERR_ARGUMENT, "invalid argument");
    auto f = std::make_unique<musg_fft>();
    f->sp.init(dim, resolutions, nb_components, -1, nullptr, true, false);
    MUSG_CUDA(cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking));
    *out = f.release();
  });
}

int musg_fft_destroy(musg_fft *fft) {
  return guard([&] { delete fft; });
}

int musg_fft_forward(musg_fft *fft, const double *in, double *out_complex) {
  return guard([&] {
    require(fft && in && out_complex, MUSG_ERR_ARGUMENT, "null argument");
    Spectral &sp = fft->sp;
    const size_t rb = (size_t)sp.g.npx * sp.ncomp * sizeof(double);
    const size_t cb = (size_t)sp.g.nk * sp.ncomp * sizeof(double2);
    if (fft->a.bytes < std::max(rb, cb)) fft->a.alloc(std::max(rb, cb));
    if (fft->b.bytes < std::max(rb, cb)) fft->b.alloc(std::max(rb, cb));
    MUSG_CUDA(cudaMemcpyAsync(fft->a.p, in, rb, cudaMemcpyHostToDevice, fft->stream));
    aos_to_soa(fft->a.as<double>(), fft->b.as<double>(), sp.ncomp, sp.g.npx, fft->stream);
    spectral_forward<double>(sp, fft->b.as<double>(), 1.0, fft->stream);
    soa_to_aos_complex((const double2 *)sp.spec64, fft->a.as<double2>(), sp.ncomp, sp.g.nk, fft->stream);
    MUSG_CUDA(cudaMemcpyAsync(out_complex, fft->a.p, cb, cudaMemcpyDeviceToHost, fft->stream));
    MUSG_CUDA(cudaStreamSynchronize(fft->stream));
  });
}

int musg_fft_inverse(musg_fft *fft, const double *in_complex, double *out) {
  return guard([&] {
    require(fft && in_complex && out, MUSG_ERR_ARGUMENT, "null argument");
    Spectral &sp = fft->sp;
    const size_t rb = (size_t)sp.g.npx * sp.ncomp * sizeof(double);
    const size_t cb = (size_t)sp.g.nk * sp.ncomp * sizeof(double2);
    if (fft->a.bytes < std::max(rb, cb)) fft->a.alloc(std::max(rb, cb));
    if (fft->b.bytes < std::max(rb, cb)) fft->b.alloc(std::max(rb, cb));
    MUSG_CUDA(cudaMemcpyAsync(fft->a.p, in_complex, cb, cudaMemcpyHostToDevice, fft->stream));
    aos_to_soa_complex(fft->a.as<double2>(), (double2 *)sp.spec64, sp.ncomp, sp.g.nk, fft->stream);
    spectral_inverse<double>(sp, fft->b.as<double>(), 1.0, fft->stream);
    soa_to_aos(fft->b.as<double>(), fft->a.as<double>(), sp.ncomp, sp.g.npx, fft->stream);
    MUSG_CUDA(cudaMemcpyAsync(out, fft->a.p, rb, cudaMemcpyDeviceToHost, fft->stream));
    MUSG_CUDA(cudaStreamSynchronize(fft->stream));
  });
}

int musg_projection_create(int dim, const int *resolutions, const double *lengths, int kind, int flags,
                           musg_projection **out) {
  return guard([&] {
    require(out && resolutions, MUSG_ERR_ARGUMENT, "null argument");
    require(kind >= 0 && kind <= 2, MUSG_ERR_ARGUMENT, "unknown projection kind");
    if (!(flags & MUSG_FLAG_ALLOW_EVEN))
      for (int d = 0; d < dim; ++d)
        require(resolutions[d] % 2 == 1, MUSG_ERR_PROJECTION,
                "Only an odd number of gridpoints in each direction is supported");
    auto p = std::make_unique<musg_projection>();
    p->kind = kind;
    p->sp.init(dim, resolutions, dim * dim, kind, lengths, (flags & MUSG_FLAG_ALLOW_EVEN) != 0, false);
    MUSG_CUDA(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    *out = p.release();
  });
}

int musg_projection_apply_noalloc(int dim, const int *resolutions, const double *lengths, int kind, int flags,
                                  const double *in_device, double *out_device, void *cuda_stream) {
  return guard([&] {
    noalloc_project(dim, resolutions, lengths, kind, flags, in_device, out_device, (cudaStream_t)cuda_stream);
  });
}

int musg_projection_destroy(musg_projection *proj) {
  return guard([&] { delete proj; });
}

int musg_projection_apply(musg_projection *proj, double *vec) {
  return guard([&] {
    require(proj && vec, MUSG_ERR_ARGUMENT, "null argument");
    Spectral &sp = proj->sp;
    const size_t rb = (size_t)sp.g.npx * sp.ncomp * sizeof(double);
    if (proj->a.bytes < rb) proj->a.alloc(rb);
    if (proj->b.bytes < rb) proj->b.alloc(rb);
    MUSG_CUDA(cudaMemcpyAsync(proj->a.p, vec, rb, cudaMemcpyHostToDevice, proj->stream));
    aos_to_soa(proj->a.as<double>(), proj->b.as<double>(), sp.ncomp, sp.g.npx, proj->stream);
    spectral_project<double>(sp, proj->b.as<double>(), proj->b.as<double>(), 1.0, proj->stream);
    soa_to_aos(proj->b.as<double>(), proj->a.as<double>(), sp.ncomp, sp.g.npx, proj->stream);
    MUSG_CUDA(cudaMemcpyAsync(vec, proj->a.p, rb, cudaMemcpyDeviceToHost, proj->stream));
    MUSG_CUDA(cudaStreamSynchronize(proj->stream));
  });
}

int musg_projection_get_operator(musg_projection *proj, double *out, long long *rows, long long *cols) {
  return guard([&] {
    require(proj, MUSG_ERR_ARGUMENT, "null projection");
    const Spectral &sp = proj->sp;
    const int dim = sp.g.dim;
    const long long nk = sp.g.nk;
    const long long nrow = proj->kind == MUSG_PROJ_FINITE_STRAIN_FAST ? dim : (long long)dim * dim * dim * dim;
    if (rows) *rows = nrow;
    if (cols) *cols = nk;
    if (!out) return;
    // the operator as the reference stores it, computed on the host from the unit
    // wave vectors (projection_small_strain.cc:56-86, projection_finite_strain.cc:62-95,
    // projection_finite_strain_fast.cc:61-73)
    int fres[3] = {sp.g.n[0], sp.g.n[1], sp.g.n[2]};
    fres[dim - 1] = sp.g.nh;
    auto freq = [](int n, int k) {
      int N = (n - 1) / 2 + 1;
      return k < N ? (double)k : (double)(-(n / 2) + k - N);
    };
    for (long long k = 0; k < nk; ++k) {
      int cc[3] = {0, 0, 0};
      long long t = k;
      for (int d = dim - 1; d >= 0; --d) {
        cc[d] = (int)(t % fres[d]);
        t /= fres[d];
      }
      double xi[3] = {0, 0, 0}, nrm = 0;
      bool zero = (k == 0);
      for (int d = 0; d < dim; ++d) {
        xi[d] = freq(sp.g.n[d], cc[d]) / sp.lengths[d];
        nrm += xi[d] * xi[d];
        if (sp.allow_even && sp.g.n[d] % 2 == 0 && cc[d] == sp.g.n[d] / 2) zero = true;
      }
      nrm = std::sqrt(nrm);
      for (int d = 0; d < dim; ++d) xi[d] = zero ? 0.0 : xi[d] / nrm;
      double *col = out + k * nrow;
      if (proj->kind == MUSG_PROJ_FINITE_STRAIN_FAST) {
        for (int d = 0; d < dim; ++d) col[d] = xi[d];
        continue;
      }
      const int D = dim, D2 = dim * dim;
      for (int m = 0; m < D; ++m)
        for (int l = 0; l < D; ++l)
          for (int j = 0; j < D; ++j)
            for (int i = 0; i < D; ++i) {
              double g;
              if (proj->kind == MUSG_PROJ_SMALL_STRAIN) {
                auto kr = [](int a, int b) { return a == b ? 1.0 : 0.0; };
                g = 0.5 * (xi[i] * kr(j, l) * xi[m] + xi[i] * kr(j, m) * xi[l] + xi[j] * kr(i, l) * xi[m] +
                           xi[j] * kr(i, m) * xi[l]) -
                    xi[i] * xi[j] * xi[l] * xi[m];
              } else {
                g = (i == l ? 1.0 : 0.0) * xi[j] * xi[m];  // outer_under(I, xi xi^T)
              }
              col[(i + D * j) + D2 * (l + D * m)] = g;
            }
    }
  });
}

}  // extern "C"
