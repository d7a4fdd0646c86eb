// Argument evaluation order of the reference's paired random draws.
//
// The reference builds its random pairs and quadruples as
//   vec2f(lcg_randomf(rng), lcg_randomf(rng))                  (hair_msnn.cu:20,212;
//   vec4f(rand1.x, rand1.y, lcg_randomf(rng), lcg_randomf(rng)) optix_common.cuh:91,140,154,161,...)
// C++ leaves the order of constructor arguments unspecified: nvcc, which
// compiles the reference's OptiX programs, evaluates them left to right
// (first draw -> x), while g++ evaluates them right to left.  To compile the
// reference's sources on the host with nvcc's order, every parenthesised
// vec2f / vec4f construction in them becomes a braced one, whose elements
// are evaluated left to right by rule (C++11 [dcl.init.list]/4).  Include
// this after hm_owl_shim.h and before the reference's sources.
#pragma once
#define vec2f(...) vec2f{__VA_ARGS__}
#define vec4f(...) vec4f{__VA_ARGS__}
