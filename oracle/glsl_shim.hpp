/*
 * glsl_shim.hpp -- the subset of GLSL 4.60 that the reference's compute shaders
 * use, as C++20 types and functions, so that the shader sources can be compiled
 * unchanged (apart from their resource declarations) and executed on the CPU.
 * TEST INFRASTRUCTURE ONLY (it builds the reference side of the parity checks).
 *
 * Semantics chosen where GLSL leaves things to the implementation:
 *   - float arithmetic is IEEE binary32, one operation at a time (compile with
 *     -ffp-contract=off); dot/length/matrix products sum left to right;
 *   - round() rounds halfway cases away from zero;
 *   - image loads outside the image return 0, stores outside are dropped;
 *   - buffer reads outside the bound range return 0, writes are dropped.
 */
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>

namespace glsl {

typedef unsigned int uint;

struct ivec1 { int x; operator int() const { return x; } };
struct ivec2 { int x, y; ivec2() : x(0), y(0) {} ivec2(int a, int b) : x(a), y(b) {} };
struct uvec3 { uint x, y, z; };
struct ivec3 {
	int x, y, z;
	ivec3() : x(0), y(0), z(0) {}
	ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
	explicit ivec3(uvec3 u) : x((int)u.x), y((int)u.y), z((int)u.z) {}
	ivec3 &operator+=(ivec3 o) { x += o.x; y += o.y; z += o.z; return *this; }
};
struct ivec4 { int x, y, z, w; };
struct uvec4 { uint x, y, z, w; };


struct vec2 {
	float x, y;
	vec2() : x(0), y(0) {}
	explicit vec2(float s) : x(s), y(s) {}
	explicit vec2(int s) : x((float)s), y((float)s) {}
	explicit vec2(bool b) : x(b ? 1.0f : 0.0f), y(b ? 1.0f : 0.0f) {}
	vec2(float a, float b) : x(a), y(b) {}
	float &operator[](int i) { return i ? y : x; }
	float operator[](int i) const { return i ? y : x; }
};

struct vec3;

/* swizzle views overlaying the storage of a vecN */
template <int A, int B, int N> struct swz2 {
	float e[N];
	operator vec2() const { return vec2(e[A], e[B]); }
	swz2 &operator=(vec2 v) { e[A] = v.x; e[B] = v.y; return *this; }
	swz2 &operator*=(vec2 v) { e[A] = e[A] * v.x; e[B] = e[B] * v.y; return *this; }
	swz2 &operator+=(vec2 v) { e[A] = e[A] + v.x; e[B] = e[B] + v.y; return *this; }
};
template <int A, int B, int C, int N> struct swz3 {
	float e[N];
	operator vec3() const;
};

struct vec3 {
	union {
		struct { float x, y, z; };
		float e[3];
		swz2<0, 1, 3> xy;
		swz2<0, 2, 3> xz;
		swz3<0, 1, 2, 3> xyz;
	};
	vec3() : x(0), y(0), z(0) {}
	explicit vec3(float s) : x(s), y(s), z(s) {}
	vec3(float a, float b, float c) : x(a), y(b), z(c) {}
	vec3(vec2 v, float c) : x(v.x), y(v.y), z(c) {}
	vec3(ivec3 v) : x((float)v.x), y((float)v.y), z((float)v.z) {}
	vec3(const vec3 &o) : x(o.x), y(o.y), z(o.z) {}
	vec3 &operator=(const vec3 &o) { x = o.x; y = o.y; z = o.z; return *this; }
	float &operator[](int i) { return e[i]; }
	float operator[](int i) const { return e[i]; }
};

struct vec4 {
	union {
		struct { float x, y, z, w; };
		float e[4];
		swz2<0, 1, 4> xy;
		swz2<2, 3, 4> zw;
		swz3<0, 1, 2, 4> xyz;
	};
	vec4() : x(0), y(0), z(0), w(0) {}
	explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
	explicit vec4(int s) : x((float)s), y((float)s), z((float)s), w((float)s) {}
	vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
	vec4(vec2 v, float c, float d) : x(v.x), y(v.y), z(c), w(d) {}
	vec4(vec3 v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
	vec4(const vec4 &o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
	vec4 &operator=(const vec4 &o) { x = o.x; y = o.y; z = o.z; w = o.w; return *this; }
	float &operator[](int i) { return e[i]; }
	float operator[](int i) const { return e[i]; }
};

template <int A, int B, int C, int N> swz3<A, B, C, N>::operator vec3() const { return vec3(e[A], e[B], e[C]); }

inline ivec3 operator+(ivec3 a, ivec3 b) { return ivec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline ivec3 operator*(ivec3 a, int s) { return ivec3(a.x * s, a.y * s, a.z * s); }


/* ---- arithmetic ---- */
inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(vec2 a, vec2 b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator*(vec2 a, vec2 b) { return vec2(a.x * b.x, a.y * b.y); }
inline vec2 operator*(vec2 a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator*(float s, vec2 a) { return vec2(s * a.x, s * a.y); }
inline vec2 operator/(vec2 a, float s) { return vec2(a.x / s, a.y / s); }
inline vec2 operator-(vec2 a) { return vec2(-a.x, -a.y); }
inline vec2 &operator+=(vec2 &a, vec2 b) { a = a + b; return a; }
inline vec2 &operator*=(vec2 &a, vec2 b) { a = a * b; return a; }

inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 &operator+=(vec3 &a, vec3 b) { a = a + b; return a; }

inline vec4 operator+(vec4 a, vec4 b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator*(float s, vec4 a) { return vec4(s * a.x, s * a.y, s * a.z, s * a.w); }
inline vec4 operator/(vec4 a, float s) { return vec4(a.x / s, a.y / s, a.z / s, a.w / s); }
inline vec4 &operator+=(vec4 &a, vec4 b) { a = a + b; return a; }

/* ---- matrices (column-major) ---- */
struct mat2 {
	vec2 c[2];
	mat2(float a, float b, float d, float e) { c[0] = vec2(a, b); c[1] = vec2(d, e); }
};
inline vec2 operator*(const mat2 &m, vec2 v)
{
	return vec2(m.c[0].x * v.x + m.c[1].x * v.y, m.c[0].y * v.x + m.c[1].y * v.y);
}

struct mat4 {
	vec4 c[4];
	mat4() {}
	mat4(float a0, float a1, float a2, float a3, float b0, float b1, float b2, float b3,
	     float c0, float c1, float c2, float c3, float d0, float d1, float d2, float d3)
	{
		c[0] = vec4(a0, a1, a2, a3); c[1] = vec4(b0, b1, b2, b3);
		c[2] = vec4(c0, c1, c2, c3); c[3] = vec4(d0, d1, d2, d3);
	}
};
inline vec4 operator*(const mat4 &m, vec4 v)
{
	vec4 r;
	for (int i = 0; i < 4; i++)
		r.e[i] = m.c[0].e[i] * v.x + m.c[1].e[i] * v.y + m.c[2].e[i] * v.z + m.c[3].e[i] * v.w;
	return r;
}
inline vec4 operator*(vec4 v, const mat4 &m)
{
	vec4 r;
	for (int j = 0; j < 4; j++)
		r.e[j] = v.x * m.c[j].x + v.y * m.c[j].y + v.z * m.c[j].z + v.w * m.c[j].w;
	return r;
}
struct mat2x4 {
	vec4 c[2];
	mat2x4(vec4 a, vec4 b) { c[0] = a; c[1] = b; }
};
inline vec2 operator*(vec4 v, const mat2x4 &m)
{
	vec2 r;
	r.x = v.x * m.c[0].x + v.y * m.c[0].y + v.z * m.c[0].z + v.w * m.c[0].w;
	r.y = v.x * m.c[1].x + v.y * m.c[1].y + v.z * m.c[1].z + v.w * m.c[1].w;
	return r;
}

/* ---- built-in functions ---- */
inline float radians(float d) { return d * 0.017453292519943295f; }
inline float cos(float a) { return ::cosf(a); }
inline float sin(float a) { return ::sinf(a); }
inline float sqrt(float a) { return ::sqrtf(a); }
inline float inversesqrt(float a) { return 1.0f / ::sqrtf(a); }
inline float abs(float a) { return ::fabsf(a); }
inline float floor(float a) { return ::floorf(a); }
inline float round(float a) { return ::roundf(a); }
inline bool  isinf(float a) { return std::isinf(a); }
inline float min(float a, float b) { return b < a ? b : a; }
inline float max(float a, float b) { return a < b ? b : a; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float modf(float x, float &ip) { ip = ::truncf(x); return x - ip; }
inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(vec2 a) { return sqrt(dot(a, a)); }
inline float length(vec3 a) { return sqrt(dot(a, a)); }
inline float distance(vec2 a, vec2 b) { return length(a - b); }
inline float distance(vec3 a, vec3 b) { return length(a - b); }

inline uint packSnorm2x16(vec2 v)
{
	int16_t a = (int16_t)::roundf(clamp(v.x, -1.0f, 1.0f) * 32767.0f);
	int16_t b = (int16_t)::roundf(clamp(v.y, -1.0f, 1.0f) * 32767.0f);
	return (uint)(uint16_t)a | ((uint)(uint16_t)b << 16);
}
inline vec2 unpackSnorm2x16(uint p)
{
	int16_t a = (int16_t)(p & 0xFFFFu), b = (int16_t)(p >> 16);
	return vec2(clamp((float)a / 32767.0f, -1.0f, 1.0f), clamp((float)b / 32767.0f, -1.0f, 1.0f));
}

/* ---- storage buffers: reads outside the bound range give 0, writes drop ---- */
template <class T> struct zero_of { static T get() { return T(); } };
template <> struct zero_of<int> { static int get() { return 0; } };
template <> struct zero_of<uint> { static uint get() { return 0; } };
template <> struct zero_of<float> { static float get() { return 0; } };

template <class T> struct ssbo {
	T *p = nullptr;
	int64_t n = 0;
	T &operator[](int64_t i)
	{
		static thread_local T sink;
		if (i >= 0 && i < n) return p[i];
		sink = zero_of<T>::get();
		return sink;
	}
};

/* ---- images ---- */
struct image1D  { const float *p = nullptr; int n = 0; int comps = 1; };  /* r32f or rg32f */
struct iimage1D { const int16_t *p = nullptr; int n = 0; };                /* r16i */
struct iimage2D { const int8_t *p = nullptr; int w = 0, h = 0; };          /* r8i */
struct image3D  { float *p = nullptr; int w = 0, h = 0, d = 0; };          /* rg32f */

inline vec4 imageLoad(const image1D &im, int i)
{
	if (i < 0 || i >= im.n) return vec4(0.0f);
	if (im.comps == 1) return vec4(im.p[i], 0.0f, 0.0f, 1.0f);
	return vec4(im.p[2 * i], im.p[2 * i + 1], 0.0f, 1.0f);
}
inline ivec4 imageLoad(const iimage1D &im, int i)
{
	if (i < 0 || i >= im.n) return ivec4{0, 0, 0, 0};
	return ivec4{im.p[i], 0, 0, 1};
}
inline ivec4 imageLoad(const iimage2D &im, ivec2 c)
{
	if (c.x < 0 || c.y < 0 || c.x >= im.w || c.y >= im.h) return ivec4{0, 0, 0, 0};
	return ivec4{im.p[c.y * im.w + c.x], 0, 0, 1};
}
inline vec4 imageLoad(const image3D &im, ivec3 c)
{
	if (c.x < 0 || c.y < 0 || c.z < 0 || c.x >= im.w || c.y >= im.h || c.z >= im.d) return vec4(0.0f);
	int64_t i = ((int64_t)c.z * im.h + c.y) * im.w + c.x;
	return vec4(im.p[2 * i], im.p[2 * i + 1], 0.0f, 1.0f);
}
inline void imageStore(image3D &im, ivec3 c, vec4 v)
{
	if (c.x < 0 || c.y < 0 || c.z < 0 || c.x >= im.w || c.y >= im.h || c.z >= im.d) return;
	int64_t i = ((int64_t)c.z * im.h + c.y) * im.w + c.x;
	im.p[2 * i] = v.x;
	im.p[2 * i + 1] = v.y;
}
inline ivec1 imageSize(const image1D &im) { return ivec1{im.n}; }
inline ivec2 imageSize(const iimage2D &im) { return ivec2(im.w, im.h); }

inline thread_local uvec3 gl_GlobalInvocationID;

} /* namespace glsl */
