// Minimal stand-in for the cpu_features header that the reference's
// src/hamming_impl.cc includes on x86 (its ext/cpu_features submodule is not
// vendored). It answers the three feature queries that file makes
// (src/hamming_impl.cc:55-73) with GCC's __builtin_cpu_supports.
// Test infrastructure only: used when compiling the reference as the oracle.
#pragma once

namespace cpu_features {

struct X86Features {
  bool sse2;
  bool avx2;
  bool avx512bw;
};

struct X86Info {
  X86Features features;
};

inline X86Info GetX86Info() {
  __builtin_cpu_init();
  X86Info info{};
  info.features.sse2 = __builtin_cpu_supports("sse2");
  info.features.avx2 = __builtin_cpu_supports("avx2");
  info.features.avx512bw = __builtin_cpu_supports("avx512bw");
  return info;
}

} // namespace cpu_features
