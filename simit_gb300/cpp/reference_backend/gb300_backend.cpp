// The GB300 backend behind the reference's backend plugin interface (see
// gb300_backend.h).  Compiled against the reference's headers.
#include "gb300_backend.h"

#include <cstring>
#include <vector>

#include "../simit.h"
#include "error.h"
#include "func.h"
#include "graph.h"
#include "ir.h"
#include "types.h"

namespace simit {
namespace backend {

namespace {

// The sets a compiled function binds: its arguments (the frontend turns a
// program's extern sets into arguments of its exported functions) and the
// externs of its environment.
std::vector<ir::Var> bindableVars(const ir::Func &func) {
  std::vector<ir::Var> out = func.getArguments();
  for (const ir::Var &v : func.getEnvironment().getExternVars()) out.push_back(v);
  return out;
}

// True when `func` binds a set `name` of `card` endpoints whose element type
// has every field of `fields`.
bool hasExternSet(const ir::Func &func, const std::string &name, size_t card,
                  const std::vector<std::string> &fields) {
  for (const ir::Var &v : bindableVars(func)) {
    if (v.getName() != name) continue;
    const ir::Type &t = v.getType();
    if (!t.isSet()) return false;
    const ir::SetType *st = t.toSet();
    const ir::UnstructuredSetType *us = st->to<ir::UnstructuredSetType>();
    if (!us || us->getCardinality() != card) return false;
    const ir::ElementType *et = st->elementType.toElement();
    for (const std::string &f : fields)
      if (!et->hasField(f)) return false;
    return true;
  }
  return false;
}

simit_gb300::FieldType facadeType(ComponentType t, const std::string &field) {
  switch (t) {
    case ComponentType::Double: return simit_gb300::FieldType::F64;
    case ComponentType::Int: return simit_gb300::FieldType::I32;
    case ComponentType::Boolean: return simit_gb300::FieldType::BOOL;
    default: break;
  }
  simit_uerror << "field " << field << ": the GB300 backend runs its programs on FP64 fields "
               << "(simit::init with 8-byte floats), int and bool fields";
  return simit_gb300::FieldType::F64;
}

// A copy of the reference set's sizes, endpoints and fields in a facade set.
std::unique_ptr<simit_gb300::Set> copySet(simit::Set *s) {
  const int card = s->getCardinality();
  std::unique_ptr<simit_gb300::Set> out =
      card ? simit_gb300::Set::edge_set(card) : std::unique_ptr<simit_gb300::Set>(
                                                    new simit_gb300::Set());
  for (Set::FieldData *f : s->getFields())
    out->add_field_raw(f->name, facadeType(f->type->getComponentType(), f->name),
                       (int)f->type->getSize());
  const int *eps = s->getEndpointsData();
  for (int e = 0; e < s->getSize(); ++e) {
    if (card) out->add_with_endpoints(reinterpret_cast<const int32_t *>(eps) + (size_t)e * card);
    else out->add();
  }
  return out;
}

// Field values between a reference set and its facade copy.
void copyFields(simit::Set *s, simit_gb300::Set *c, bool toFacade) {
  for (Set::FieldData *f : s->getFields()) {
    simit_gb300::FieldData *d = c->field(f->name);
    const size_t bytes = (size_t)s->getSize() * f->sizeOfType;
    simit_iassert(d && d->data.size() == bytes);
    if (bytes == 0) continue;
    if (toFacade) std::memcpy(d->data.data(), f->data, bytes);
    else std::memcpy(f->data, d->data.data(), bytes);
  }
}

}  // namespace

std::string gb300ProgramOf(const ir::Func &func) {
  const std::string name = func.getName();
  if (hasExternSet(func, "points", 0, {"x", "v", "m", "fixed"}) &&
      hasExternSet(func, "springs", 2, {"k", "l0"}))
    return name == "timestep" ? "isprings_app" : (name == "main" ? "isprings" : "");
  if (hasExternSet(func, "points", 0, {"b", "c"}) && hasExternSet(func, "springs", 2, {"a"}))
    return name == "main" ? "cg" : "";
  if (hasExternSet(func, "verts", 0, {"x", "v", "c", "m"}) &&
      hasExternSet(func, "tets", 4, {"u", "l", "W", "B"}))
    return name == "initializeTet" ? "femTet.init" : (name == "main" ? "femTet" : "");
  return "";
}

Function *GB300Backend::compile(ir::Func func, const ir::Storage &) {
  const std::string prog = gb300ProgramOf(func);
  if (prog.empty()) {
    std::string sets;
    for (const ir::Var &v : bindableVars(func))
      sets += (sets.empty() ? "" : ", ") + v.getName();
    simit_uerror << "the GB300 backend runs the programs of the sparse-system path "
                 << "(isprings, cg, femTet); " << func.getName() << " (binding: " << sets
                 << ") is not one of them";
  }
  return new GB300Function(func, prog);
}

GB300Function::GB300Function(const ir::Func &func, const std::string &program)
    : Function(func), program_(program) {
  const bool fem = program_.rfind("femTet", 0) == 0;
  vname_ = fem ? "verts" : "points";
  ename_ = fem ? "tets" : "springs";
}

GB300Function::~GB300Function() {}

void GB300Function::bind(const std::string &name, simit::Set *set) {
  if (name == vname_) V_ = set;
  else if (name == ename_) E_ = set;
  else simit_uerror << "no set " << name << " in " << program_;
  initialized_ = false;
}

void GB300Function::bind(const std::string &name, void *) {
  simit_uerror << program_ << " takes no tensor argument " << name;
}

void GB300Function::bind(const std::string &name, TensorData &) {
  simit_uerror << program_ << " takes no sparse tensor argument " << name;
}

void GB300Function::convertSets() {
  simit_uassert(V_ && E_) << "bind " << vname_ << " and " << ename_ << " first";
  fv_ = copySet(V_);
  fe_ = copySet(E_);
}

Function::FuncType GB300Function::init() {
  convertSets();
  try {
    core_.reset(new simit_gb300::Function(program_));
    core_->bind(vname_, fv_.get());
    core_->bind(ename_, fe_.get());
    core_->init();
  } catch (const simit_gb300::SimitException &e) {
    core_.reset();
    simit_uerror << "GB300 backend: " << e.what();
  }
  initialized_ = true;
  simit_gb300::Function *core = core_.get();
  return [core]() {
    try {
      core->run();
    } catch (const simit_gb300::SimitException &e) {
      simit_uerror << "GB300 backend: " << e.what();
    }
  };
}

bool GB300Function::isInitialized() { return initialized_; }

void GB300Function::copyIn() {
  copyFields(V_, fv_.get(), true);
  copyFields(E_, fe_.get(), true);
}

void GB300Function::copyOut() {
  copyFields(V_, fv_.get(), false);
  copyFields(E_, fe_.get(), false);
}

void GB300Function::unmapArgs(bool updated) {
  if (!updated || !core_) return;
  copyIn();
  try {
    core_->unmapArgs(true);
  } catch (const simit_gb300::SimitException &e) {
    simit_uerror << "GB300 backend: " << e.what();
  }
}

void GB300Function::mapArgs() {
  if (!core_) return;
  try {
    core_->mapArgs();
  } catch (const simit_gb300::SimitException &e) {
    simit_uerror << "GB300 backend: " << e.what();
  }
  copyOut();
}

void GB300Function::print(std::ostream &os) const {
  os << "GB300 backend: program " << program_ << " over " << vname_ << " and " << ename_
     << " (libsimit_gb300 C ABI, sm_103a kernels)";
  // the device-side copies of the bound sets, once init has made them
  if (!fv_ || !fe_) return;
  simit_gb300::Set *sets[2] = {fv_.get(), fe_.get()};
  const std::string names[2] = {vname_, ename_};
  for (int k = 0; k < 2; ++k) {
    simit_gb300::Set *c = sets[k];
    os << "; " << names[k] << " " << c->getSize();
    if (c->getCardinality()) os << "x" << c->getCardinality();
    os << " [";
    for (int i = 0; i < c->numFields(); ++i)
      os << (i ? " " : "") << c->field_at(i).name << ":" << c->field_at(i).comps;
    os << "]";
    if (c->getCardinality()) {
      os << " endpoints";
      for (int32_t e : c->endpoints()) os << " " << e;
    }
  }
}

void GB300Function::printMachine(std::ostream &os) const {
  os << "GB300 backend: the kernels are precompiled in libsimit_gb300.so for sm_103a";
}

}  // namespace backend
}  // namespace simit
