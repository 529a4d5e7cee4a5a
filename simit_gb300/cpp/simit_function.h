// simit_gb300::Function: bind / init / run / runSafe / mapArgs / unmapArgs
// over the built-in programs (see simit.h).  Included by simit.h.
#pragma once

namespace simit_gb300 {

class DevBuf {
 public:
  DevBuf() = default;
  explicit DevBuf(size_t bytes) { alloc(bytes); }
  ~DevBuf() { release(); }
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  void alloc(size_t bytes) {
    release();
    bytes_ = bytes;
    check_cuda(cudaMalloc(&p_, bytes < 256 ? 256 : bytes), "cudaMalloc");
  }
  void release() {
    if (p_) cudaFree(p_);
    p_ = nullptr;
  }
  void *get() const { return p_; }
  template <typename T> T *as() const { return reinterpret_cast<T *>(p_); }
  size_t bytes() const { return bytes_; }

 private:
  void *p_ = nullptr;
  size_t bytes_ = 0;
};

class Function {
 public:
  explicit Function(const std::string &program, int device = 0) : prog_(program), dev_(device) {
    static const char *known[] = {"isprings", "isprings_app", "cg", "femTet", "femTet.init"};
    for (const char *k : known)
      if (program == k) defined_ = true;
  }
  ~Function() {
    if (solver_) sg_solver_destroy(solver_);
    if (ctx_) sg_ctx_destroy(ctx_);
  }
  Function(const Function &) = delete;
  Function &operator=(const Function &) = delete;

  bool defined() const { return defined_; }

  // Function::bind(name, Set*) (src/function.cpp:92-114): unknown names are an error.
  void bind(const std::string &name, Set *set) {
    if (!defined_) throw SimitException("Function::bind: undefined function " + prog_);
    const bool ok = (vertex_name() == name) || (edge_name() == name);
    if (!ok) throw SimitException("Function::bind: no argument named " + name + " in " + prog_);
    (name == vertex_name() ? V_ : E_) = set;
    initialized_ = false;
  }

  // Pattern build, device buffers and the solver (src/backend/llvm/
  // llvm_function.cpp:248-465 builds its indices and temporaries here).
  void init() {
    if (!V_ || !E_) throw SimitException("Function::init: bind both sets first");
    check(sg_ctx_create(dev_, &ctx_), "sg_ctx_create");
    n_ = V_->getSize();
    nE_ = E_->getSize();
    card_ = E_->getCardinality();
    ep_.alloc((size_t)nE_ * card_ * 4);
    check_cuda(cudaMemcpy(ep_.get(), E_->endpoints().data(), (size_t)nE_ * card_ * 4,
                          cudaMemcpyHostToDevice), "endpoints");
    ve_ptr_.alloc((size_t)(n_ + 1) * 4);
    ve_idx_.alloc((size_t)nE_ * card_ * 4);
    rowptr_.alloc((size_t)(n_ + 1) * 4);
    check(sg_incidence_build(ctx_, n_, ep_.as<int32_t>(), nE_, card_, ve_ptr_.as<uint32_t>(),
                             ve_idx_.as<uint32_t>()), "sg_incidence_build");
    int64_t nnzb = 0;
    check(sg_pattern_count(ctx_, n_, ep_.as<int32_t>(), nE_, card_, ve_ptr_.as<uint32_t>(),
                           ve_idx_.as<uint32_t>(), rowptr_.as<uint32_t>(), &nnzb),
          "sg_pattern_count");
    colidx_.alloc((size_t)nnzb * 4);
    check(sg_pattern_fill(ctx_, n_, ep_.as<int32_t>(), nE_, card_, ve_ptr_.as<uint32_t>(),
                          ve_idx_.as<uint32_t>(), rowptr_.as<uint32_t>(),
                          colidx_.as<uint32_t>()), "sg_pattern_fill");
    int32_t maxrow = 0;
    check(sg_pattern_maxrow(ctx_, n_, rowptr_.as<uint32_t>(), &maxrow), "sg_pattern_maxrow");
    mesh_ = sg_mesh{n_, card_, nE_, ep_.as<int32_t>(), ve_ptr_.as<uint32_t>(),
                    ve_idx_.as<uint32_t>(), rowptr_.as<uint32_t>(), colidx_.as<uint32_t>(),
                    nnzb, maxrow};
    const int bs = prog_ == "cg" ? 1 : 3;
    vals_.alloc((size_t)nnzb * bs * bs * 8);
    rhs_.alloc((size_t)n_ * bs * 8);
    tmp_.alloc((size_t)n_ * bs * 8);
    // device mirrors of every field of both sets
    for (Set *s : {V_, E_})
      for (int i = 0;; ++i) {
        FieldData *f = field_by_index(s, i);
        if (!f) break;
        dev_fields_[key(s, f->name)].alloc(f->data.size());
      }
    if (prog_ != "femTet.init") {
      sg_matrix A{n_, bs, nnzb, rowptr_.as<uint32_t>(), colidx_.as<uint32_t>(), SG_F64,
                  vals_.get()};
      sg_solve_opts o{};
      o.precision = SG_SOLVE_F64;
      o.precond = SG_PRECOND_NONE;
      o.verify = 0;
      if (prog_ == "isprings") { o.stop = SG_STOP_NORMR2; o.tol = 1e-5; o.maxiters = 25; }
      if (prog_ == "isprings_app") { o.stop = SG_STOP_NORMR2; o.tol = 1e-12; o.maxiters = 50; }
      if (prog_ == "cg") { o.stop = SG_STOP_NORMR; o.tol = 1e-6; o.maxiters = 5; }
      if (prog_ == "femTet") { o.stop = SG_STOP_NORMR2; o.tol = 1e-6; o.maxiters = 100; }
      check(sg_solver_create(ctx_, &A, &o, &solver_), "sg_solver_create");
    }
    initialized_ = true;
  }
  bool isInitialized() const { return initialized_; }

  // Copy the bound sets' fields to the device (the reference's unmapArgs
  // pushes host data to the GPU: src/backend/gpu/gpu_function.cpp:181-197).
  void unmapArgs(bool updated = true) {
    if (!updated) return;
    for (Set *s : {V_, E_})
      for (int i = 0;; ++i) {
        FieldData *f = field_by_index(s, i);
        if (!f) break;
        check_cuda(cudaMemcpy(dev_fields_[key(s, f->name)].get(), f->data.data(), f->data.size(),
                              cudaMemcpyHostToDevice), "unmapArgs");
      }
  }
  // Copy the fields the program writes back to the host (the reference's
  // mapArgs pulls them: src/backend/gpu/gpu_function.cpp:174-179).
  void mapArgs() {
    for (auto &w : written()) {
      Set *s = w.first == 0 ? V_ : E_;
      FieldData *f = s->field(w.second);
      if (!f) continue;
      check(sg_ctx_sync(ctx_), "sync");
      check_cuda(cudaMemcpy(f->data.data(), dev_fields_[key(s, f->name)].get(), f->data.size(),
                            cudaMemcpyDeviceToHost), "mapArgs");
    }
  }

  void run() {
    if (!initialized_) throw SimitException("Function::run: call init() first");
    if (prog_ == "isprings" || prog_ == "isprings_app") run_isprings(prog_ == "isprings" ? 1 : 0);
    else if (prog_ == "cg") run_cg();
    else if (prog_ == "femTet.init") run_femtet_init();
    else run_femtet();
    check(sg_ctx_sync(ctx_), "run");
  }

  // Function::runSafe (src/function.cpp:121-129): init if needed, push the
  // arguments (unmapArgs), run, pull the results (mapArgs).
  void runSafe() {
    if (!initialized_) init();
    unmapArgs(true);
    run();
    mapArgs();
  }

  sg_solve_result lastSolve() const { return res_; }

 private:
  std::string vertex_name() const {
    return prog_.rfind("femTet", 0) == 0 ? "verts" : "points";
  }
  std::string edge_name() const { return prog_.rfind("femTet", 0) == 0 ? "tets" : "springs"; }
  static std::string key(Set *s, const std::string &n) {
    return std::to_string((uintptr_t)s) + ":" + n;
  }
  static FieldData *field_by_index(Set *s, int i) {
    return i < s->numFields() ? &s->field_at(i) : nullptr;
  }
  void *dev(Set *s, const char *name) {
    auto it = dev_fields_.find(key(s, name));
    if (it == dev_fields_.end()) throw SimitException(std::string("missing field ") + name);
    return it->second.get();
  }
  std::vector<std::pair<int, std::string>> written() const {
    if (prog_ == "isprings" || prog_ == "isprings_app") return {{0, "x"}, {0, "v"}};
    if (prog_ == "cg") return {{0, "c"}};
    if (prog_ == "femTet.init") return {{0, "m"}, {1, "B"}, {1, "W"}};
    return {{0, "x"}, {0, "v"}};
  }

  void run_isprings(int form) {
    const double h = 1e-2;
    const double viscous = form == 1 ? 1e-1 : 2.0;
    const double grav_test[3] = {0.0, 0.0, -9.81}, grav_app[3] = {0.0, -9.81, 0.0};
    void *x = dev(V_, "x"), *v = dev(V_, "v");
    check(sg_assemble_springs(ctx_, &mesh_, SG_F64, form, x, v, dev(V_, "m"),
                              (const uint8_t *)dev(V_, "fixed"), dev(E_, "k"), dev(E_, "l0"), h,
                              viscous, form == 1 ? grav_test : grav_app, vals_.get(), rhs_.get(),
                              1),
          "sg_assemble_springs");
    check(sg_solver_refresh(solver_), "sg_solver_refresh");
    check(sg_solver_solve(solver_, rhs_.as<double>(), (double *)v, &res_), "sg_solver_solve");
    check(sg_axpy(ctx_, (int64_t)n_ * 3, SG_F64, h, v, x), "sg_axpy");
  }

  void run_cg() {
    check(sg_assemble_scalar_springs(ctx_, &mesh_, SG_F64, dev(E_, "a"), 1.0, -0.01, vals_.get(), 1),
          "sg_assemble_scalar_springs");
    void *c = dev(V_, "c");
    check_cuda(cudaMemset(c, 0, (size_t)n_ * 8), "memset");
    check(sg_solver_refresh(solver_), "sg_solver_refresh");
    check(sg_solver_solve(solver_, (const double *)dev(V_, "b"), (double *)c, &res_),
          "sg_solver_solve");
  }

  void run_femtet_init() {
    check(sg_tet_precompute(ctx_, &mesh_, SG_F64, dev(V_, "x"), 1000.0, dev(E_, "B"),
                            dev(E_, "W"), dev(V_, "m")),
          "sg_tet_precompute");
  }

  void run_femtet() {
    const double h = 0.01, rho = 1000.0, grav[3] = {0.0, -10.0, 0.0};
    void *x = dev(V_, "x"), *v = dev(V_, "v");
    const int32_t *c = (const int32_t *)dev(V_, "c");
    check(sg_assemble_tet_force(ctx_, &mesh_, SG_F64, SG_MODEL_NEOHOOKEAN, x, v, c, dev(E_, "B"),
                                dev(E_, "W"), dev(E_, "u"), dev(E_, "l"), h, rho, grav,
                                rhs_.get(), 1),
          "sg_assemble_tet_force");
    check(sg_assemble_tet_stiffness(ctx_, &mesh_, SG_F64, SG_MODEL_NEOHOOKEAN, x, c,
                                    dev(E_, "B"), dev(E_, "W"), dev(E_, "u"), dev(E_, "l"), h,
                                    rho, vals_.get(), 1),
          "sg_assemble_tet_stiffness");
    check_cuda(cudaMemcpy(tmp_.get(), v, (size_t)n_ * 24, cudaMemcpyDeviceToDevice), "copy");
    check(sg_solver_refresh(solver_), "sg_solver_refresh");
    check(sg_solver_solve(solver_, rhs_.as<double>(), tmp_.as<double>(), &res_),
          "sg_solver_solve");
    check_cuda(cudaMemcpy(v, tmp_.get(), (size_t)n_ * 24, cudaMemcpyDeviceToDevice), "copy");
    check(sg_axpy(ctx_, (int64_t)n_ * 3, SG_F64, h, tmp_.get(), x), "sg_axpy");
  }

  std::string prog_;
  int dev_ = 0;
  bool defined_ = false, initialized_ = false;
  Set *V_ = nullptr, *E_ = nullptr;
  sg_ctx *ctx_ = nullptr;
  sg_solver *solver_ = nullptr;
  sg_mesh mesh_{};
  int32_t n_ = 0, card_ = 0;
  int64_t nE_ = 0;
  DevBuf ep_, ve_ptr_, ve_idx_, rowptr_, colidx_, vals_, rhs_, tmp_;
  std::map<std::string, DevBuf> dev_fields_;
  sg_solve_result res_{};
};

}  // namespace simit_gb300
