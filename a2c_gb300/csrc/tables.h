// Geometry of the mixed form's FP32 tables (shared by the kernels and the
// host code that builds and checks them).
#pragma once

namespace a2c {

constexpr double kTabR0 = 1.0;    // pair tables: r in [1, 7) A ...
constexpr double kTabInvH = 160.0;  // ... h = 1/160 A (knots on the 5.0 / 5.05 A branch points)
constexpr int kTabN = 960;
constexpr double kEmbInvH = 64.0;   // embedding tables: rho in [0, 64), h = 1/64
constexpr int kEmbN = 4096;

}  // namespace a2c
