// Velocity and position integration of rigid bodies, shared by the host
// World (csrc/host/novaphy_host.cpp, which runs its contact solve between
// the two) and the serving loop's coupled scenes, whose bodies step on the
// device as free bodies without contacts (csrc/pbf_boundary.cu), so that
// every caller integrates with the same float operations: semi-implicit Euler as in
// src/dynamics/integrator.cpp:20-60,
//   v += (g + f / m) dt,  w += I^-1 t dt,  w *= 0.999,
//   x += v dt,  q += 0.5 dt (w, 0) * q, then q normalised.
// Quaternions are (w, x, y, z); inv_inertia is row-major 3x3.  No contraction
// is assumed: host code is built with -ffp-contract=off, and the device copy
// is compiled with -fmad=false and IEEE division and square root.
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define PBF_RIGID_HD __host__ __device__
#else
#define PBF_RIGID_HD
#endif

namespace pbf_rigid {

PBF_RIGID_HD inline float rigid_sqrt(float x) {
#if defined(__CUDA_ARCH__)
    return sqrtf(x);
#else
    return std::sqrt(x);
#endif
}

PBF_RIGID_HD inline void integrate_velocity(float v[3], float w[3], const float g[3],
                                            const float f[3], float inv_mass, const float ii[9],
                                            const float t[3], float dt) {
    for (int d = 0; d < 3; ++d) v[d] += (g[d] + f[d] * inv_mass) * dt;
    const float it0 = ii[0] * t[0] + (ii[1] * t[1] + ii[2] * t[2]);
    const float it1 = ii[3] * t[0] + (ii[4] * t[1] + ii[5] * t[2]);
    const float it2 = ii[6] * t[0] + (ii[7] * t[1] + ii[8] * t[2]);
    w[0] += it0 * dt;
    w[1] += it1 * dt;
    w[2] += it2 * dt;
    for (int d = 0; d < 3; ++d) w[d] = w[d] * 0.999f;
}

PBF_RIGID_HD inline void integrate_position(float p[3], float q[4], const float v[3],
                                            const float w[3], float dt) {
    for (int d = 0; d < 3; ++d) p[d] += v[d] * dt;
    const float qw = q[0], qx = q[1], qy = q[2], qz = q[3];
    const float dw = 0.5f * (-w[0] * qx - w[1] * qy - w[2] * qz);
    const float dx = 0.5f * (w[0] * qw + w[2] * qy - w[1] * qz);
    const float dy = 0.5f * (w[1] * qw - w[2] * qx + w[0] * qz);
    const float dz = 0.5f * (w[2] * qw + w[1] * qx - w[0] * qy);
    float nw = qw + dw * dt, nx = qx + dx * dt, ny = qy + dy * dt, nz = qz + dz * dt;
    const float n = rigid_sqrt((nw * nw + nx * nx) + (ny * ny + nz * nz));
    if (n > 0.0f) {
        nw = nw / n;
        nx = nx / n;
        ny = ny / n;
        nz = nz / n;
    }
    q[0] = nw;
    q[1] = nx;
    q[2] = ny;
    q[3] = nz;
}

}  // namespace pbf_rigid
