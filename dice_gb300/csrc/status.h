// Status codes and the exception type used inside the library; the C-ABI
// converts them to int return codes (include/shci_gpu.h).
#pragma once
#include <stdexcept>
#include <string>

namespace shci {

enum Status : int {
  kOk = 0,
  kErrInvalid = 1,
  kErrIO = 2,
  kErrCuda = 3,
  kErrOOM = 4,
  kErrNoConv = 5,
  kErrTimeout = 6,
  kErrState = 7,
};

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

constexpr int kMaxOrbitals = 64;

}  // namespace shci
