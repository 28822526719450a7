// ref_philox_kat.cpp -- test infrastructure.  Runs the reference's own
// Random123/philox.h (RayFactorCL/Random123/philox.h:259-326, the generator that
// RayFactorCL/RayFactorGPU.cl:1,486-499 calls) on counter/key pairs read from
// stdin ("c0 c1 c2 c3 k0 k1" in hex per line) and prints the four output words
// in hex.  Its output pins the oracle's and the CUDA library's Philox.
#include <cstdio>
#include <cstdint>
#include <Random123/philox.h>

int main()
{
    unsigned c0, c1, c2, c3, k0, k1;
    while (std::scanf("%x %x %x %x %x %x", &c0, &c1, &c2, &c3, &k0, &k1) == 6) {
        philox4x32_ctr_t c = {{c0, c1, c2, c3}};
        philox4x32_key_t k = {{k0, k1}};
        philox4x32_ctr_t r = philox4x32(c, k);
        std::printf("%08x %08x %08x %08x\n", r.v[0], r.v[1], r.v[2], r.v[3]);
    }
    return 0;
}
