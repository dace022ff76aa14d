// pt_jit.h — kernels compiled at run time for GLSL SDF snippets (pt_jit.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "kernel/pt_megakernel.h"

// One PT_SDF_CUSTOM slot: its translation, functions named <prefix>sdf and
// <prefix>sdfmaterial.
struct JitSlot {
    int slot = 0;
    std::string prefix;
    std::string code;
};

// What a module holds: the megakernel (kernel[0] without, kernel[1] with
// path traces), the wavefront engine's march kernel (kernel[0]), or the
// FP64 reference renderer's megakernel (kernel[0], kernel[1] as for the
// megakernel; the snippets compiled with every GLSL float a double).  Each
// is its own NVRTC program, compiled when first needed.
enum JitKind { kJitMegakernel = 0, kJitMarch = 1, kJitFp64 = 2, kJitKinds = 3 };
constexpr int kJitMaxKernels = 2;

struct JitModule {
    std::string key;  // the program text it was compiled from
    cudaLibrary_t lib = nullptr;
    cudaKernel_t kernel[kJitMaxKernels] = {nullptr, nullptr};
};

int pt_jit_translate_slot(const char* source, int slot, JitSlot& out, std::string& err);
std::string pt_jit_program(const std::vector<JitSlot>& slots, JitKind kind);
// Compiles for the compute capability of `device` (pt_jit_compile) or for
// sm (e.g. 103) and returns the cubin and the kernels' lowered names.
// contract: compile with FMA contraction (--fmad=true) instead of the
// shader's separate roundings.
int pt_jit_compile(int device, const std::string& program, JitKind kind, std::vector<char>& cubin,
                   std::string lowered[kJitMaxKernels], std::string& log, bool contract = false);
int pt_jit_compile_for(int sm, const std::string& program, JitKind kind, std::vector<char>& cubin,
                       std::string lowered[kJitMaxKernels], std::string& log, bool contract = false);
int pt_jit_load(const std::vector<char>& cubin, JitKind kind, const std::string lowered[kJitMaxKernels], JitModule& m,
                std::string& err);
void pt_jit_unload(JitModule& m);
// The megakernel of a kJitMegakernel or kJitFp64 module over the dispatch in params.
cudaError_t pt_jit_launch(const JitModule& m, const KParams* params, bool trace, cudaStream_t stream);
