// Metal Shading Language surface for compiling the reference's per-Gaussian
// helper functions and kernel bodies as plain C++ on the host — TEST
// INFRASTRUCTURE ONLY (it pins the oracle to the reference's own source; see
// ref_kernels.cpp and ref_build.py).
//
// Provided: the vector types the helpers use (float2/3/4, int2/3, uint2/3)
// with component-wise arithmetic; float2x2 and float3x3 stored as columns
// (m[c] is column c, m[c][r] its row r; the n-scalar constructor fills
// column by column, the one-scalar constructor makes a diagonal); matrix
// products evaluated as sums over k in increasing order, each product
// rounded before it is added (the translation unit is compiled with
// -ffp-contract=off); the MSL functions they call (min, max, clamp, exp,
// sqrt, rsqrt, ceil, dot, normalize, transpose, fma, as_type, clz, atomics,
// threadgroup barriers and the SIMD-group reductions, on host threads); and
// empty address-space qualifiers (threadgroup storage: see below).
//
// Two choices are made where MSL leaves the bits open: exp() calls the
// function installed by ref_set_expf (the oracle's det_expf on both sides of
// a bit-exact comparison; libm's expf when none is installed), and
// rsqrt(x) is 1/sqrt(x), correctly rounded twice - the same choices as the
// oracle's float path.  The Metal compiler's fast-math contractions are not
// reproduced: this compiles the source's written arithmetic, in IEEE order.
#pragma once

// standard headers first: the address-space macros below would rewrite them
#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <thread>
#include <type_traits>
#include <vector>

typedef uint32_t uint;
namespace mshim {
using HostThread = std::thread;   // named before `thread` becomes an address-space macro
}
typedef uint8_t uchar;

#define device
#define constant
#define thread
#define threadgroup

namespace mshim {

using ExpFn = float (*)(float);
extern ExpFn g_expf;

template <class T> struct vec2 {
    T x, y;
    vec2() : x(0), y(0) {}
    vec2(T a, T b) : x(a), y(b) {}
    explicit vec2(T a) : x(a), y(a) {}
    template <class U> explicit vec2(const vec2<U> &o) : x((T)o.x), y((T)o.y) {}
    T &operator[](int i) { return i == 0 ? x : y; }
    const T &operator[](int i) const { return i == 0 ? x : y; }
};
template <class T> struct vec3 {
    T x, y, z;
    vec3() : x(0), y(0), z(0) {}
    vec3(T a, T b, T c) : x(a), y(b), z(c) {}
    explicit vec3(T a) : x(a), y(a), z(a) {}
    template <class U> explicit vec3(const vec3<U> &o) : x((T)o.x), y((T)o.y), z((T)o.z) {}
    T &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> struct vec4 {
    T x, y, z, w;
    vec4() : x(0), y(0), z(0), w(0) {}
    vec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    explicit vec4(T a) : x(a), y(a), z(a), w(a) {}
};

#define MSHIM_V2OP(op)                                                                                  \
    template <class T> inline vec2<T> operator op(vec2<T> a, vec2<T> b) { return {a.x op b.x, a.y op b.y}; } \
    template <class T> inline vec2<T> operator op(vec2<T> a, T s) { return {a.x op s, a.y op s}; }           \
    template <class T> inline vec2<T> operator op(T s, vec2<T> a) { return {s op a.x, s op a.y}; }
#define MSHIM_V3OP(op)                                                                                  \
    template <class T> inline vec3<T> operator op(vec3<T> a, vec3<T> b) {                                  \
        return {a.x op b.x, a.y op b.y, a.z op b.z};                                                        \
    }                                                                                                      \
    template <class T> inline vec3<T> operator op(vec3<T> a, T s) { return {a.x op s, a.y op s, a.z op s}; } \
    template <class T> inline vec3<T> operator op(T s, vec3<T> a) { return {s op a.x, s op a.y, s op a.z}; }
MSHIM_V2OP(+) MSHIM_V2OP(-) MSHIM_V2OP(*) MSHIM_V2OP(/)
MSHIM_V3OP(+) MSHIM_V3OP(-) MSHIM_V3OP(*) MSHIM_V3OP(/)
#undef MSHIM_V2OP
#undef MSHIM_V3OP
template <class T> inline vec3<T> operator-(vec3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline vec3<T> &operator+=(vec3<T> &a, vec3<T> b) { a = a + b; return a; }
template <class T> inline vec3<T> &operator*=(vec3<T> &a, T s) { a = a * s; return a; }

// Square matrices stored as columns.
template <int N> struct fmat {
    using col_t = typename std::conditional<N == 2, vec2<float>, vec3<float>>::type;
    col_t c[N];
    fmat() {}
    explicit fmat(float d) {
        for (int i = 0; i < N; i++)
            for (int j = 0; j < N; j++) set(i, j, i == j ? d : 0.f);
    }
    template <class... A, class = typename std::enable_if<sizeof...(A) == N * N>::type>
    fmat(A... a) {
        const float v[N * N] = {(float)a...};
        for (int i = 0; i < N; i++)
            for (int j = 0; j < N; j++) set(i, j, v[i * N + j]);
    }
    col_t &operator[](int i) { return c[i]; }
    const col_t &operator[](int i) const { return c[i]; }
    float get(int col, int row) const { return ((const float *)&c[col])[row]; }
    void set(int col, int row, float v) { ((float *)&c[col])[row] = v; }
};
static_assert(sizeof(vec2<float>) == 8 && sizeof(vec3<float>) == 12, "packed vectors");

template <int N> inline fmat<N> operator*(const fmat<N> &a, const fmat<N> &b) {
    fmat<N> r;
    for (int j = 0; j < N; j++)
        for (int i = 0; i < N; i++) {
            float s = a.get(0, i) * b.get(j, 0);
            for (int k = 1; k < N; k++) s = s + a.get(k, i) * b.get(j, k);
            r.set(j, i, s);
        }
    return r;
}
template <int N> inline fmat<N> operator+(const fmat<N> &a, const fmat<N> &b) {
    fmat<N> r;
    for (int j = 0; j < N; j++)
        for (int i = 0; i < N; i++) r.set(j, i, a.get(j, i) + b.get(j, i));
    return r;
}
template <int N, class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
inline fmat<N> operator*(S s, const fmat<N> &a) {
    fmat<N> r;
    for (int j = 0; j < N; j++)
        for (int i = 0; i < N; i++) r.set(j, i, (float)s * a.get(j, i));
    return r;
}
template <int N> inline fmat<N> transpose(const fmat<N> &a) {
    fmat<N> r;
    for (int j = 0; j < N; j++)
        for (int i = 0; i < N; i++) r.set(j, i, a.get(i, j));
    return r;
}

}  // namespace mshim

typedef mshim::vec2<float> float2;
typedef mshim::vec3<float> float3;
typedef mshim::vec4<float> float4;
typedef mshim::vec2<int> int2;
typedef mshim::vec3<int> int3;
typedef mshim::vec2<uint> uint2;
typedef mshim::vec3<uint> uint3;
typedef mshim::fmat<2> float2x2;
typedef mshim::fmat<3> float3x3;
using mshim::transpose;

inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline uint min(uint a, uint b) { return a < b ? a : b; }
inline uint max(uint a, uint b) { return a > b ? a : b; }
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float3 clamp(float3 v, float lo, float hi) { return {clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi)}; }
inline float exp(float x) { return mshim::g_expf ? mshim::g_expf(x) : std::exp(x); }
inline float3 exp(float3 v) { return {exp(v.x), exp(v.y), exp(v.z)}; }
inline float sqrt(float x) { return std::sqrt(x); }
inline float rsqrt(float x) { return 1.f / std::sqrt(x); }
inline float ceil(float x) { return std::ceil(x); }
inline float log(float x) { return std::log(x); }
inline float cos(float x) { return std::cos(x); }
inline float sin(float x) { return std::sin(x); }
inline float fma(float a, float b, float c) { return std::fma(a, b, c); }
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float3 normalize(float3 v) { return v * rsqrt(dot(v, v)); }
inline float saturate(float x) { return min(max(x, 0.f), 1.f); }
inline uint clz(uint x) { return x ? (uint)__builtin_clz(x) : 32u; }
template <class To, class From> inline To as_type(From f) {
    static_assert(sizeof(To) == sizeof(From), "as_type size");
    To t;
    std::memcpy(&t, &f, sizeof(t));
    return t;
}

inline float fabs(float x) { return std::fabs(x); }
inline float3 max(float3 v, float s) { return {max(v.x, s), max(v.y, s), max(v.z, s)}; }
inline float3 fma(float3 a, float b, float3 c) { return {fma(a.x, b, c.x), fma(a.y, b, c.y), fma(a.z, b, c.z)}; }
inline float3 fma(float3 a, float3 b, float3 c) { return {fma(a.x, b.x, c.x), fma(a.y, b.y, c.y), fma(a.z, b.z, c.z)}; }
inline float3 saturate(float3 v) { return {saturate(v.x), saturate(v.y), saturate(v.z)}; }

// Device atomics: every read-modify-write under one lock (threadgroups are
// emulated by host threads, see below).
namespace mshim {
std::mutex &atomic_lock();
}
typedef uint atomic_uint;
typedef float atomic_float;
enum mshim_memory_order { memory_order_relaxed };
inline uint atomic_fetch_add_explicit(atomic_uint *p, uint v, mshim_memory_order) {
    std::lock_guard<std::mutex> lk(mshim::atomic_lock());
    const uint o = *p;
    *p = o + v;
    return o;
}
inline float atomic_fetch_add_explicit(atomic_float *p, float v, mshim_memory_order) {
    std::lock_guard<std::mutex> lk(mshim::atomic_lock());
    const float o = *p;
    *p = o + v;
    return o;
}

// Threadgroups on host threads.  A kernel that uses threadgroup memory,
// threadgroup barriers or SIMD-group functions runs each threadgroup as one
// host thread per GPU thread; its `threadgroup` arrays become function
// statics (groups run one after another, so one copy serves each group),
// threadgroup_barrier is a barrier of the group's threads, and a SIMD group
// is 32 consecutive threads of the group whose simd_* calls meet at a
// barrier of their own (the reference calls them from all lanes).  simd_sum
// adds the lanes in lane order.
namespace mshim {
struct HostBarrier {
    int n = 0;
    std::atomic<int> waiting{0};
    std::atomic<uint32_t> generation{0};
    void wait() {
        const uint32_t gen = generation.load(std::memory_order_acquire);
        if (waiting.fetch_add(1, std::memory_order_acq_rel) + 1 == n) {
            waiting.store(0, std::memory_order_relaxed);
            generation.fetch_add(1, std::memory_order_acq_rel);
            generation.notify_all();
        } else {
            while (generation.load(std::memory_order_acquire) == gen) generation.wait(gen, std::memory_order_acquire);
        }
    }
};
struct SimdGroup {
    HostBarrier bar;
    alignas(16) unsigned char slot[2][32][16];
};
struct GroupState {
    HostBarrier bar;
    SimdGroup sg[32];
};
extern GroupState *g_group;
extern thread_local int t_lane, t_sg;
extern thread_local unsigned t_simd_op;

// One exchange per SIMD-group call: every lane writes its value, meets the
// others at the barrier, then reduces.  Consecutive calls alternate between
// two slot sets, so one barrier per call suffices (a lane can only reuse a
// set after every lane has passed the next call's barrier).
template <class T, class F> inline T simd_exchange(const T &v, F reduce) {
    static_assert(sizeof(T) <= 16, "simd value size");
    SimdGroup &sg = g_group->sg[t_sg];
    unsigned char (*slot)[16] = sg.slot[t_simd_op++ & 1u];
    std::memcpy(slot[t_lane], &v, sizeof(T));
    sg.bar.wait();
    return reduce(slot);
}
template <class T> inline T lane_value(const unsigned char (*slot)[16], int lane) {
    T v;
    std::memcpy(&v, slot[lane], sizeof(T));
    return v;
}
}  // namespace mshim

namespace mem_flags {
enum { mem_none = 0, mem_threadgroup = 1, mem_device = 2 };
}
inline void threadgroup_barrier(int) { mshim::g_group->bar.wait(); }
inline float simd_sum(float v) {
    return mshim::simd_exchange(v, [](const unsigned char (*sl)[16]) {
        float s = mshim::lane_value<float>(sl, 0);
        for (int l = 1; l < 32; l++) s = s + mshim::lane_value<float>(sl, l);
        return s;
    });
}
inline int simd_max(int v) {
    return mshim::simd_exchange(v, [](const unsigned char (*sl)[16]) {
        int s = mshim::lane_value<int>(sl, 0);
        for (int l = 1; l < 32; l++) s = max(s, mshim::lane_value<int>(sl, l));
        return s;
    });
}
inline int simd_or(int v) {
    return mshim::simd_exchange(v, [](const unsigned char (*sl)[16]) {
        int s = 0;
        for (int l = 0; l < 32; l++) s |= mshim::lane_value<int>(sl, l);
        return s;
    });
}
template <class T> inline T simd_broadcast(T v, int lane) {
    return mshim::simd_exchange(v, [lane](const unsigned char (*sl)[16]) { return mshim::lane_value<T>(sl, lane); });
}
