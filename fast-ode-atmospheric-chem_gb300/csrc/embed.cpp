// The relocatable integrator of the generated variant (generated.cu, compiled
// to a cubin by the build before this file) embedded in the library, so that
// jit.cpp can link it with each mechanism's generated code.
#ifndef FO_GENERATED_RDC
#error "FO_GENERATED_RDC must name the relocatable cubin of generated.cu"
#endif

__asm__(".section .rodata\n"
        ".balign 64\n"
        ".globl fo_generated_rdc_begin\n"
        ".hidden fo_generated_rdc_begin\n"
        "fo_generated_rdc_begin:\n"
        ".incbin \"" FO_GENERATED_RDC "\"\n"
        ".globl fo_generated_rdc_end\n"
        ".hidden fo_generated_rdc_end\n"
        "fo_generated_rdc_end:\n"
        ".previous\n");
