// simit_gb300::Map: a user's `map f to E reduce +` on facade Sets, with the
// element function given as CUDA C++ source -- the element_block (system
// matrix result) or element_vector (system vector result) that
// simit_gb300.simfront.compile_map writes from a .sim function, or one
// written by hand -- compiled at run time (sg_jit_assembly_create /
// sg_jit_vector_create).  It opens the facade to programs beyond the
// built-in ones of Function: bind the element set and the vertex set, name
// the fields in the source's f[] order, init() and run().  Included by
// simit.h.
//
//   Map m(source, /*bs=*/3, /*vector=*/false, {"element:B", "vertex:x"});
//   m.bind(&tets, &verts);       // a map over the vertices: bind(&verts, &verts)
//   m.init();                    // pattern, compile, device buffers
//   m.run();                     // fields to the device, assemble, values back
//   m.values();                  // [nnzb*bs*bs] on m.rowptr() / m.colidx(), or [n*bs]
#pragma once

namespace simit_gb300 {

class Map {
 public:
  Map(const std::string &element_source, int bs, bool vector_result,
      std::vector<std::string> fields, bool fp64 = true, bool exact = true, int device = 0)
      : src_(element_source), bs_(bs), vec_(vector_result), fields_(std::move(fields)),
        fp64_(fp64), exact_(exact), dev_(device) {
    if (fields_.size() > 8) throw SimitException("Map: at most 8 fields");
    for (const std::string &f : fields_)
      if (f.rfind("element:", 0) != 0 && f.rfind("vertex:", 0) != 0)
        throw SimitException("Map: field " + f + " is not element:<name> or vertex:<name>");
  }
  ~Map() {
    if (jit_) sg_jit_assembly_destroy(jit_);
    if (ctx_) sg_ctx_destroy(ctx_);
  }
  Map(const Map &) = delete;
  Map &operator=(const Map &) = delete;

  // The element set and the vertex set its endpoints index; for a map over
  // the vertices themselves pass the vertex set twice.
  void bind(Set *elements, Set *vertices) {
    E_ = elements;
    V_ = vertices;
    initialized_ = false;
  }

  void init() {
    if (!E_ || !V_) throw SimitException("Map::init: bind the sets first");
    if (!ctx_) check(sg_ctx_create(dev_, &ctx_), "sg_ctx_create");
    n_ = V_->getSize();
    const bool over_vertices = E_ == V_ || E_->getCardinality() == 0;
    card_ = over_vertices ? 1 : E_->getCardinality();
    nE_ = over_vertices ? n_ : E_->getSize();
    std::vector<int32_t> ep(over_vertices ? (size_t)n_ : E_->endpoints().size());
    if (over_vertices)
      for (int32_t i = 0; i < n_; ++i) ep[i] = i;
    else
      ep = E_->endpoints();
    for (int32_t v : ep)
      if (v < 0 || v >= n_) throw SimitException("Map::init: endpoint outside the vertex set");
    ep_.alloc(ep.size() * 4);
    check_cuda(cudaMemcpy(ep_.get(), ep.data(), ep.size() * 4, cudaMemcpyHostToDevice),
               "endpoints");
    ve_ptr_.alloc((size_t)(n_ + 1) * 4);
    ve_idx_.alloc(ep.size() * 4);
    rowptr_d_.alloc((size_t)(n_ + 1) * 4);
    check(sg_incidence_build(ctx_, n_, ep_.as<int32_t>(), nE_, card_, ve_ptr_.as<uint32_t>(),
                             ve_idx_.as<uint32_t>()), "sg_incidence_build");
    int64_t nnzb = 0;
    check(sg_pattern_count(ctx_, n_, ep_.as<int32_t>(), nE_, card_, ve_ptr_.as<uint32_t>(),
                           ve_idx_.as<uint32_t>(), rowptr_d_.as<uint32_t>(), &nnzb),
          "sg_pattern_count");
    colidx_d_.alloc((size_t)nnzb * 4);
    check(sg_pattern_fill(ctx_, n_, ep_.as<int32_t>(), nE_, card_, ve_ptr_.as<uint32_t>(),
                          ve_idx_.as<uint32_t>(), rowptr_d_.as<uint32_t>(),
                          colidx_d_.as<uint32_t>()), "sg_pattern_fill");
    int32_t maxrow = 0;
    check(sg_pattern_maxrow(ctx_, n_, rowptr_d_.as<uint32_t>(), &maxrow), "sg_pattern_maxrow");
    mesh_ = sg_mesh{n_, card_, nE_, ep_.as<int32_t>(), ve_ptr_.as<uint32_t>(),
                    ve_idx_.as<uint32_t>(), rowptr_d_.as<uint32_t>(), colidx_d_.as<uint32_t>(),
                    nnzb, maxrow};
    rowptr_.resize(n_ + 1);
    colidx_.resize(nnzb);
    check_cuda(cudaMemcpy(rowptr_.data(), rowptr_d_.get(), rowptr_.size() * 4,
                          cudaMemcpyDeviceToHost), "rowptr");
    if (nnzb)
      check_cuda(cudaMemcpy(colidx_.data(), colidx_d_.get(), colidx_.size() * 4,
                            cudaMemcpyDeviceToHost), "colidx");
    if (!jit_) {
      const int dt = fp64_ ? SG_F64 : SG_F32;
      check(vec_ ? sg_jit_vector_create(ctx_, src_.c_str(), card_, bs_, dt, exact_, &jit_)
                 : sg_jit_assembly_create(ctx_, src_.c_str(), card_, bs_, dt, exact_, &jit_),
            "Map: compiling the element function");
    }
    const size_t nvals = vec_ ? (size_t)n_ * bs_ : (size_t)nnzb * bs_ * bs_;
    vals_d_.alloc(nvals * (fp64_ ? 8 : 4));
    vals_.assign(nvals, 0.0);
    dfields_.clear();
    for (size_t k = 0; k < fields_.size(); ++k) dfields_.emplace_back(new DevBuf());
    initialized_ = true;
  }

  // Fields to the device (floating-point ones in the map's precision), the
  // assembly, the values back to the host.
  void run() {
    if (!initialized_) init();
    std::vector<const void *> ptrs(fields_.size());
    for (size_t k = 0; k < fields_.size(); ++k) {
      const bool elem = fields_[k].rfind("element:", 0) == 0;
      const std::string name = fields_[k].substr(elem ? 8 : 7);
      Set *s = elem ? E_ : V_;
      FieldData *f = s->field(name);
      if (!f) throw SimitException("Map::run: no field " + fields_[k]);
      std::vector<unsigned char> host;
      const std::vector<unsigned char> *src = &f->data;
      if (f->type == FieldType::F64 && !fp64_) {
        host.resize(f->data.size() / 2);
        for (size_t i = 0; i < f->data.size() / 8; ++i)
          reinterpret_cast<float *>(host.data())[i] =
              (float)reinterpret_cast<const double *>(f->data.data())[i];
        src = &host;
      } else if (f->type == FieldType::F32 && fp64_) {
        host.resize(f->data.size() * 2);
        for (size_t i = 0; i < f->data.size() / 4; ++i)
          reinterpret_cast<double *>(host.data())[i] =
              reinterpret_cast<const float *>(f->data.data())[i];
        src = &host;
      }
      dfields_[k]->alloc(src->size());
      if (!src->empty())
        check_cuda(cudaMemcpy(dfields_[k]->get(), src->data(), src->size(),
                              cudaMemcpyHostToDevice), "fields");
      ptrs[k] = dfields_[k]->get();
    }
    check(vec_ ? sg_jit_assemble_vector(jit_, &mesh_, ptrs.data(), (int32_t)ptrs.size(),
                                        vals_d_.get())
               : sg_jit_assemble(jit_, &mesh_, ptrs.data(), (int32_t)ptrs.size(), vals_d_.get()),
          "Map::run");
    check(sg_ctx_sync(ctx_), "Map::run");
    if (fp64_) {
      check_cuda(cudaMemcpy(vals_.data(), vals_d_.get(), vals_.size() * 8,
                            cudaMemcpyDeviceToHost), "values");
    } else {
      std::vector<float> tmp(vals_.size());
      check_cuda(cudaMemcpy(tmp.data(), vals_d_.get(), tmp.size() * 4, cudaMemcpyDeviceToHost),
                 "values");
      for (size_t i = 0; i < tmp.size(); ++i) vals_[i] = tmp[i];
    }
  }

  // The reference's name for init-if-needed, push, run, pull.
  void runSafe() { run(); }

  const std::vector<double> &values() const { return vals_; }
  const std::vector<uint32_t> &rowptr() const { return rowptr_; }
  const std::vector<uint32_t> &colidx() const { return colidx_; }
  // The device values and pattern, for a solver or an SpMV through the C ABI.
  const sg_mesh &mesh() const { return mesh_; }
  void *device_values() const { return vals_d_.get(); }
  sg_ctx *context() const { return ctx_; }

 private:
  std::string src_;
  int bs_;
  bool vec_;
  std::vector<std::string> fields_;
  bool fp64_, exact_;
  int dev_;
  bool initialized_ = false;
  Set *E_ = nullptr, *V_ = nullptr;
  sg_ctx *ctx_ = nullptr;
  sg_jit_assembly *jit_ = nullptr;
  sg_mesh mesh_{};
  int32_t n_ = 0, card_ = 0;
  int64_t nE_ = 0;
  DevBuf ep_, ve_ptr_, ve_idx_, rowptr_d_, colidx_d_, vals_d_;
  std::vector<std::unique_ptr<DevBuf>> dfields_;
  std::vector<uint32_t> rowptr_, colidx_;
  std::vector<double> vals_;
};

}  // namespace simit_gb300
