// The GB300 backend behind the reference's own backend plugin interface:
// simit::backend::BackendImpl (src/backend/backend_impl.h:16-23) and
// simit::backend::Function (src/backend/backend_function.h:27-88).
//
// This is the reference-side binding: it is compiled against the reference's
// headers and linked with the reference's frontend, IR and lowering, so that
// a Simit program loaded with simit::Program (src/program.cpp:101-107) and
// bound and run through simit::Function (src/function.cpp:22-139) reaches
// libsimit_gb300's C ABI.  The backend serves the programs of the
// sparse-system path -- the ones whose assembly and solve the library
// implements -- recognised from the compiled function's name and its extern
// sets (isprings main and timestep, cg main, femTet main and initializeTet);
// any other program is refused with a user error.  Each recognised program
// runs on the library's host facade (simit_gb300/cpp/simit.h), which holds
// the device copies of the bound sets' fields.
#pragma once

#include <memory>
#include <ostream>
#include <string>

#include "backend/backend_function.h"
#include "backend/backend_impl.h"

namespace simit_gb300 {
class Function;
class Set;
}  // namespace simit_gb300

namespace simit {
namespace backend {

/// The program of the sparse-system path that `func` is, or "" when it is
/// none of them.
std::string gb300ProgramOf(const ir::Func &func);

class GB300Backend : public BackendImpl {
 public:
  /// A GB300Function for a program of the path; a user error otherwise.
  Function *compile(ir::Func func, const ir::Storage &storage) override;
};

class GB300Function : public Function {
 public:
  GB300Function(const ir::Func &func, const std::string &program);
  ~GB300Function() override;

  /// Keeps the set; its fields are copied to the device at init and at
  /// every unmapArgs.
  void bind(const std::string &name, simit::Set *set) override;
  /// Tensor and sparse-tensor arguments: the path's programs take none.
  void bind(const std::string &name, void *data) override;
  void bind(const std::string &name, TensorData &data) override;

  /// Builds the pattern, the device buffers and the solver (the work of
  /// LLVMFunction::init and initIndices, src/backend/llvm/
  /// llvm_function.cpp:248-465); the returned function runs one call of
  /// the program on the GPU.
  FuncType init() override;
  bool isInitialized() override;

  /// Pulls the fields the program writes back into the bound sets
  /// (GPUFunction::mapArgs, src/backend/gpu/gpu_function.cpp:174-179).
  void mapArgs() override;
  /// Pushes the bound sets' fields to the device (GPUFunction::unmapArgs,
  /// src/backend/gpu/gpu_function.cpp:181-197).
  void unmapArgs(bool updated = true) override;

  void print(std::ostream &os) const override;
  void printMachine(std::ostream &os) const override;

  const std::string &program() const { return program_; }
  /// The facade's copies of the bound sets, as init builds them (for
  /// checks of the conversion).
  const simit_gb300::Set *vertexCopy() const { return fv_.get(); }
  const simit_gb300::Set *elementCopy() const { return fe_.get(); }
  /// Builds the facade's copies of the bound sets without touching the
  /// device (init does this first).
  void convertSets();

 private:
  void copyIn();
  void copyOut();

  std::string program_, vname_, ename_;
  simit::Set *V_ = nullptr, *E_ = nullptr;
  std::unique_ptr<simit_gb300::Set> fv_, fe_;
  std::unique_ptr<simit_gb300::Function> core_;
  bool initialized_ = false;
};

}  // namespace backend
}  // namespace simit
