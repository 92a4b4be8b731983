// xoshiro256+ streams on the host: seeding (splitmix64, srcs/random.hpp:32-91)
// and arbitrary skip-ahead.
//
// The reference gives OpenMP thread t the stream `seed` advanced by t jump()s and
// lets each thread consume it sample by sample (srcs/feynman_integral.hpp:85-93);
// with one thread, sample i therefore uses draws [i(2E-1), (i+1)(2E-1)) of the
// seed's stream (every sample takes exactly 2E-1 uniforms,
// srcs/tropical_sampling.hpp:479,557).  The GPU reproduces exactly that stream:
// each lane starts at its first sample's offset.  The state update is linear over
// GF(2), so advancing by k steps is a 256x256 bit matrix T^k applied to the state;
// the 64 matrices T^(2^b) are built once per process and shipped to the device,
// where a lane composes the ones for the set bits of its offset.
#pragma once

#include <cstdint>
#include <vector>

namespace ft {

struct xstate {
    uint64_t s[4];
};

xstate seed_state(uint64_t seed);
uint64_t next(xstate& x);

// 64 matrices T^(2^b), b = 0..63; matrix b, column c (the image of state bit c) is
// words [(b*256 + c)*4, +4)
const std::vector<uint64_t>& power_table();

// T^steps x
xstate advance(xstate x, uint64_t steps);

}  // namespace ft
