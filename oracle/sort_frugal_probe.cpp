// sort_frugal_probe.cpp -- TEST INFRASTRUCTURE.  Compiled by oracle/Makefile
// against the reference's own tools/sort_points/Sort_Frugal sources (their
// main.cpp with its entry point renamed, and unsuck_platform_specific.cpp)
// into oracle/_ref/libsfref.so, so the CPU tests can pin the Morton order of
// the product's cloud builder to the reference's splitBy3 /
// mortonEncode_magicbits (Sort_Frugal/src/main.cpp:58-77).
#define main sort_frugal_main
#include "main.cpp"
#undef main

extern "C" uint64_t sfref_morton(uint32_t x, uint32_t y, uint32_t z) {
    return mortonEncode_magicbits(x, y, z);
}
