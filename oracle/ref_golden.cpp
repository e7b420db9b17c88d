// ref_golden.cpp -- golden-vector generator linked against the reference's own
// primitives, compiled from the sources where they lie in the reference tree
// (oracle/Makefile, target "ref").  TEST INFRASTRUCTURE: it pins the oracle
// restatement; nothing in the product links it.
//
// Reference pieces used (compiled, not copied):
//   MathUtil::xxhash32 / Bernoulli     src/core/math/MathUtil.hpp:179-228
//   UniformSampler (PCG32)             src/core/sampling/UniformSampler.hpp:22-75
//   rand_normal_2 / sample_standard_normal  src/core/sampling/Gaussian.cpp:23-35,89-104
//   TangentFrame(n)                    src/core/math/TangentFrame.hpp:74-98
//
// Output: one JSON document on stdout.  Floats are printed as the decimal of
// their bit pattern (uint32) so the files compare bit-exactly.
#include "math/MathUtil.hpp"
#include "math/TangentFrame.hpp"
#include "sampling/Gaussian.hpp"
#include "sampling/UniformSampler.hpp"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

using namespace Tungsten;

static uint32_t bits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static uint64_t bits64(double d) { uint64_t u; std::memcpy(&u, &d, 8); return u; }

// Deterministic input stream for the generator itself (splitmix64).
static uint64_t sm_state = 0x5EED5EEDull;
static uint64_t sm_next() {
    uint64_t z = (sm_state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

template <typename F>
static void list(const char *name, int n, F &&item, bool last = false) {
    std::printf("\"%s\": [", name);
    for (int i = 0; i < n; ++i) {
        if (i) std::printf(",");
        std::printf("\n  ");
        item(i);
    }
    std::printf("\n]%s\n", last ? "" : ",");
}

int main() {
    std::printf("{\n");
    // xxhash32 of one, two and four words.
    list("xxhash32_1", 64, [](int) {
        uint32_t x = uint32_t(sm_next());
        std::printf("[%u, %u]", x, MathUtil::xxhash32(x));
    });
    list("xxhash32_2", 64, [](int i) {
        uint32_t x = i < 8 ? uint32_t(i - 4) : uint32_t(sm_next()), y = uint32_t(sm_next());
        std::printf("[%u, %u, %u]", x, y, MathUtil::xxhash32(Vec2u(x, y)));
    });
    list("xxhash32_4", 64, [](int) {
        uint32_t a = uint32_t(sm_next()), b = uint32_t(sm_next()), c = uint32_t(sm_next()), d = uint32_t(sm_next());
        std::printf("[%u, %u, %u, %u, %u]", a, b, c, d, MathUtil::xxhash32(Vec4u(a, b, c, d)));
    });
    // PCG streams after set_state(s): 12 next1D floats (bit patterns).
    list("pcg_next1d", 32, [](int i) {
        uint64_t s = i < 4 ? uint64_t(i) : (i < 8 ? (sm_next() & 0xFFFFFFFFull) : sm_next());
        UniformSampler u;
        u.set_state(s);
        std::printf("[\"%llu\"", (unsigned long long)s);
        for (int k = 0; k < 12; ++k) std::printf(", %u", bits(u.next1D()));
        std::printf("]");
    });
    // cell1D impulse lists: set_state(xxhash32(Vec2u(cell, seed)) + 1u), then
    // N x (position next1D, weight Bernoulli(next1D, -1, 1, 0.5)).
    list("cell1d", 48, [](int i) {
        uint32_t cell = i < 6 ? uint32_t(i - 3) : uint32_t(sm_next() % 4096u);
        uint32_t seed = i < 24 ? uint32_t(1 + i) : uint32_t(sm_next());
        const unsigned N = 8;
        UniformSampler u;
        u.set_state(MathUtil::xxhash32(Vec2u(cell, seed)) + 1u);
        std::printf("[%u, %u, [", cell, seed);
        for (unsigned k = 0; k < N; ++k) {
            float t = u.next1D();
            float w = MathUtil::Bernoulli(u.next1D(), -1.f, 1.f, 0.5f);
            std::printf("%s%u, %u", k ? ", " : "", bits(t), bits(w));
        }
        std::printf("]]");
    });
    // cell3D impulse lists: set_state(xxhash32(Vec4u(k, j, i, seed)) + 1u), then
    // N x (Vec3f(sampler.next3D()), Bernoulli(next1D)) as this compiler orders next3D.
    list("cell3d", 32, [](int n) {
        int ci = int(sm_next() % 64u) - 32, cj = int(sm_next() % 64u) - 32, ck = int(sm_next() % 64u) - 32;
        uint32_t seed = n < 16 ? uint32_t(1 + n) : uint32_t(sm_next());
        const unsigned N = 8;
        UniformSampler u;
        Vec3u ijk = Vec3u(Vec3i(ci, cj, ck));
        u.set_state(MathUtil::xxhash32(Vec4u(ijk.z(), ijk.y(), ijk.x(), seed)) + 1u);
        std::printf("[%d, %d, %d, %u, [", ci, cj, ck, seed);
        for (unsigned k = 0; k < N; ++k) {
            Vec3f p = Vec3f(u.next3D());
            float w = MathUtil::Bernoulli(u.next1D(), -1.f, 1.f, 0.5f);
            std::printf("%s%u, %u, %u, %u", k ? ", " : "", bits(p.x()), bits(p.y()), bits(p.z()), bits(w));
        }
        std::printf("]]");
    });
    // Box-Muller pairs: sampler.set_state(s); sample_standard_normal(4, sampler).
    list("normal4", 32, [](int) {
        uint32_t s = uint32_t(sm_next());
        UniformSampler u;
        u.set_state(s);
        Eigen::VectorXd z = sample_standard_normal(4, u);
        std::printf("[%u, \"%llu\", \"%llu\", \"%llu\", \"%llu\"]", s,
                    (unsigned long long)bits64(z(0)), (unsigned long long)bits64(z(1)),
                    (unsigned long long)bits64(z(2)), (unsigned long long)bits64(z(3)));
    });
    // TangentFrame(n) of unnormalized directions.
    list("tangent_frame", 48, [](int i) {
        float v[3];
        for (int c = 0; c < 3; ++c) v[c] = float(int(sm_next() % 20001u) - 10000) / 977.0f;
        if (i == 0) { v[0] = 0.f; v[1] = 0.f; v[2] = 1.f; }
        if (i == 1) { v[0] = 0.f; v[1] = 0.f; v[2] = -1.f; }
        if (i == 2) { v[0] = 1.f; v[1] = 0.f; v[2] = 0.f; }
        if (i == 3) { v[0] = -1.f; v[1] = 0.f; v[2] = 0.f; }
        TangentFrame f(Vec3f(v[0], v[1], v[2]));
        std::printf("[%u, %u, %u, %u, %u, %u, %u, %u, %u, %u, %u, %u]", bits(v[0]), bits(v[1]), bits(v[2]),
                    bits(f.tangent.x()), bits(f.tangent.y()), bits(f.tangent.z()),
                    bits(f.bitangent.x()), bits(f.bitangent.y()), bits(f.bitangent.z()),
                    bits(f.normal.x()), bits(f.normal.y()), bits(f.normal.z()));
    });
    // Known answer of RaySegmentBatchTest.cpp:44-65,144-175: the seeded 1D noise at
    // coordinate 5.001 / (lengthScale * 0.7071067811865475f) with radius 3 and
    // 3 impulses per cell, built from the reference sampler and hash.
    list("se_noise_1d_seeds", 73, [](int i) {
        const float radius = 3.0f;
        const unsigned impulses = 3;
        const float coordinate = 5.001f / (1.0f * 0.7071067811865475f);
        const uint32_t seed = uint32_t(123 + i);
        const float grid = coordinate / radius;
        const float cellFloor = std::floor(grid);
        const int cell = int(cellFloor);
        const float fraction = grid - cellFloor;
        double sum = 0;
        UniformSampler u;
        for (int offset = -1; offset <= 1; ++offset) {
            u.set_state(MathUtil::xxhash32(Vec2u(uint32_t(cell + offset), seed)) + 1U);
            for (unsigned k = 0; k < impulses; ++k) {
                const float impulse = u.next1D();
                const float weight = u.next1D() < 0.5f ? -1.0f : 1.0f;
                const double d = (double(fraction) - offset - impulse) * radius;
                if ((fraction - offset - impulse) * (fraction - offset - impulse) < 1.0f)
                    sum += weight * std::exp(-0.5 * d * d);
            }
        }
        const double value = sum / std::sqrt(double(impulses) / radius * std::sqrt(M_PI));
        std::printf("[%u, \"%llu\"]", seed, (unsigned long long)bits64(value));
    }, true);
    std::printf("}\n");
    return 0;
}
