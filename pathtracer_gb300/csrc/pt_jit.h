// pt_jit.h — run-time compiled megakernels for GLSL SDF snippets (pt_jit.cu).
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

struct JitModule {
    std::string key;  // the program text it was compiled from
    cudaLibrary_t lib = nullptr;
    cudaKernel_t kernel[2] = {nullptr, nullptr};  // megakernel without / with traces
};

int pt_jit_translate_slot(const char* source, int slot, JitSlot& out, std::string& err);
std::string pt_jit_program(const std::vector<JitSlot>& slots);
int pt_jit_compile(int device, const std::string& program, std::vector<char>& cubin, std::string lowered[2],
                   std::string& log);
int pt_jit_compile_for(int sm, const std::string& program, std::vector<char>& cubin, std::string lowered[2],
                       std::string& log);
int pt_jit_load(const std::vector<char>& cubin, const std::string lowered[2], JitModule& m, std::string& err);
void pt_jit_unload(JitModule& m);
cudaError_t pt_jit_launch(const JitModule& m, const KParams* params, bool trace, cudaStream_t stream);
