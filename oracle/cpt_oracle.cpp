/*
 * cpt_oracle.cpp — TEST INFRASTRUCTURE ONLY: the FP64 CPU oracle.
 *
 * A restatement, in plain C++ and double precision, of CudaPathTracing's path-tracing
 * hot path: Morton keys, sort, Karras hierarchy emission, refit, closest-hit traversal,
 * primitive intersection, BSDFs, camera and the STATIC render loop.  Every function cites
 * the reference file:line it follows and keeps the reference's order of floating-point
 * operations, so that (built with -ffp-contract=off) it reproduces the reference's own
 * code, compiled here by oracle/Makefile into oracle/_ref, bit for bit.  The config
 * estimator (Lambertian, IOR, media, depth limits) has no reference code; it is restated
 * here from the same formulas as the CUDA kernels.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library,
 * and only as a checker or as the timed CPU baseline; the product never does.
 */
#include "cpt.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

#define ORC_API extern "C" __attribute__((visibility("default")))

namespace orc {

static const double INF = 999999.0;                 // rtmath.cuh:8
static const double PI = 3.14159265358979323846;    // rtmath.cuh:9

// ------------------------------------------------------------------ vector maths
// rtmath.cuh:17-112; each helper keeps the reference's evaluation order.
struct V3 { double x, y, z; };
static inline V3 v3(double x, double y, double z) { V3 r = {x, y, z}; return r; }
static inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
static inline V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline V3 operator*(double t, V3 v) { return v3(v.x * t, v.y * t, v.z * t); }
static inline V3 operator*(V3 v, double t) { return v3(v.x * t, v.y * t, v.z * t); }
static inline V3 operator/(V3 v, double t) { return v3(v.x / t, v.y / t, v.z / t); }
static inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double len2(V3 v) { return v.x * v.x + v.y * v.y + v.z * v.z; }
static inline double length(V3 v) { return std::sqrt(len2(v)); }
static inline V3 unit(V3 v) { return v / length(v); }
static inline V3 cross(V3 a, V3 b)
{
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline double mmin(double a, double b) { return a < b ? a : b; }   // rtmath.cuh:11
static inline double mmax(double a, double b) { return a > b ? a : b; }   // rtmath.cuh:12

// Complex helpers used by the conductor Fresnel term (rtmath.cuh:179-225).
struct C2 { double x, y; };
static inline C2 c2(double x, double y) { C2 r = {x, y}; return r; }
static inline C2 cdiv(C2 a, C2 b)
{
    double den = b.x * b.x + b.y * b.y;
    return c2((a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den);
}
static inline double cnorm(C2 v) { return v.x * v.x + v.y * v.y; }

// ------------------------------------------------------------------ RNG
// PCG32 (O'Neill 2014), the stand-in for curand (Render.cu:28-32): stream = pixel offset.
struct Rng {
    uint64_t state, inc;
    uint32_t next()
    {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((0u - rot) & 31u));
    }
    void init(uint64_t seed, uint64_t stream)
    {
        state = 0u;
        inc = (stream << 1u) | 1u;
        next();
        state += seed;
        next();
    }
    double uniform() { return ((double)next() + 1.0) * (1.0 / 4294967296.0); }   // (0, 1]
    // delta draws ahead in O(log delta) (LCG jump-ahead, Brown 1994)
    void advance(uint64_t delta)
    {
        uint64_t cm = 6364136223846793005ULL, cp = inc, am = 1, ap = 0;
        while (delta) {
            if (delta & 1u) {
                am *= cm;
                ap = ap * cm + cp;
            }
            cp *= cm + 1;
            cm *= cm;
            delta >>= 1;
        }
        state = am * state + ap;
    }
};

// Config estimator: sample k of a pixel uses the pixel's stream k * 2^32 draws ahead; sample
// radiance is summed in groups of sampleGroup(spp) samples, group sums added in order.
static int sampleGroup(int spp) { return spp <= 256 ? 8 : (spp + 31) / 32; }

// ------------------------------------------------------------------ scene objects
enum MatType { M_NONE = 0, M_LIGHT = 1, M_OPAQUE = 2, M_SPEC = 3, M_ROUGH = 4, M_VOLUME = 5, M_LAMBERT = 6 };

struct Material {                       // Material.cuh:5-22
    V3 color;
    double ax, ay;
    int type;
    double eta;                         // 1.51 under the reference estimator (Material.cuh:12)
    double sigma_t, albedo;
};

struct HitRecord {                      // HitRecord.cuh:5-30
    V3 hitPos = {0, 0, 0};
    V3 hitColor = {-1, -1, -1};
    V3 hitWm = {0, 0, 0};
    V3 normal = {0, 0, 0};
    const Material* material = nullptr;
    double t = INF;
    bool frontFace = false;
};

struct Ray { V3 o, d; };
static inline V3 at(const Ray& r, double t) { return r.o + t * r.d; }   // Ray.cuh:19

static inline void setFaceNormal(HitRecord& rec, const Ray& ray, V3 outward)   // HitRecord.cuh:32-36
{
    rec.frontFace = dot(ray.d, outward) < 0;
    rec.normal = rec.frontFace ? outward : -outward;
}

struct Box { V3 mn, mx; };
static inline Box boxOf(V3 p0, V3 p1)   // AABB.cuh:12-20
{
    Box b;
    b.mn = v3(mmin(p0.x, p1.x), mmin(p0.y, p1.y), mmin(p0.z, p1.z));
    b.mx = v3(mmax(p0.x, p1.x), mmax(p0.y, p1.y), mmax(p0.z, p1.z));
    return b;
}
static inline Box boxUnion(const Box& a, const Box& b)   // AABB.cuh:21-29
{
    Box r;
    r.mn = v3(mmin(a.mn.x, b.mn.x), mmin(a.mn.y, b.mn.y), mmin(a.mn.z, b.mn.z));
    r.mx = v3(mmax(a.mx.x, b.mx.x), mmax(a.mx.y, b.mx.y), mmax(a.mx.z, b.mx.z));
    return r;
}
static inline Box pad(Box b)   // AABB.cuh:30-40
{
    const double delta = 0.0001;
    b.mn.x -= delta; b.mn.y -= delta; b.mn.z -= delta;
    b.mx.x += delta; b.mx.y += delta; b.mx.z += delta;
    return boxOf(b.mn, b.mx);
}

enum Kind { K_LIGHT, K_SPHERE, K_TRI };

struct Prim {
    Kind kind;
    V3 center;          // Hittable::center
    Box box;            // Hittable::aabb
    Material mat;
    // sphere (Hittable.cuh:10-26)
    V3 sc; double r;
    // light (Hittable.cuh:346-366)
    double lw, lh; V3 ln, eu, ev; bool visible;
    // triangle (Hittable.cuh:57-83)
    V3 p0, p1, p2, n0, n1, n2;
    double uv[6];                  // uv0, uv1, uv2
    const uint8_t* tex;            // RGB8 texture or NULL (Triangle::texture)
    int texW, texH;
};

// Nearest texel (HitRecord::sampleTexture, HitRecord.cuh:38-49; Camera::getSkyBox, Camera.cuh:56-61):
// x = min(max(int(u * width), 0), width - 1), likewise y, texels / 255.  int(x) of a double
// outside the int range is undefined in C++; it is taken as saturating here, as on the GPU.
static inline int texIndex(double x, int n)
{
    double f = x * (double)n;
    int i = f >= 2147483647.0 ? 2147483647 : (f <= -2147483648.0 ? (-2147483647 - 1) : (f != f ? 0 : (int)f));
    return i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
}
static inline V3 texel(const uint8_t* img, int w, int h, double u, double v)
{
    int x = texIndex(u, w), y = texIndex(v, h);
    const uint8_t* q = img + 3 * ((size_t)y * w + x);
    return v3(q[0] / 255.0, q[1] / 255.0, q[2] / 255.0);
}

static Prim makeLight(const cpt_light& L)   // Light ctor Hittable.cuh:359-365; Hittable(Light) :424-454
{
    Prim p;
    p.kind = K_LIGHT;
    p.sc = v3(L.center[0], L.center[1], L.center[2]);
    p.lw = L.width;
    p.lh = L.height;
    p.visible = L.visible != 0;
    p.mat.color = v3(L.color[0], L.color[1], L.color[2]);
    p.mat.ax = 1.0; p.mat.ay = 1.0; p.mat.type = M_LIGHT; p.mat.eta = 1.51;
    p.mat.sigma_t = 0; p.mat.albedo = 0;
    V3 n = v3(L.normal[0], L.normal[1], L.normal[2]);
    p.ln = unit(n);
    p.eu = std::fabs(p.ln.x) > 0.9 ? unit(cross(v3(0, 1, 0), p.ln)) : unit(cross(v3(1, 0, 0), p.ln));
    p.ev = unit(cross(p.ln, p.eu));
    p.center = p.sc;
    // Hittable(Light): the box of the four corners, padded.
    V3 N = unit(p.ln);
    V3 T = std::fabs(N.x) > 0.9 ? unit(cross(v3(0, 1, 0), N)) : unit(cross(v3(1, 0, 0), N));
    V3 B = unit(cross(N, T));
    V3 c[4] = {
        p.sc + T * (p.lw / 2) + B * (p.lh / 2),
        p.sc + T * (p.lw / 2) + B * (-p.lh / 2),
        p.sc + T * (-p.lw / 2) + B * (p.lh / 2),
        p.sc + T * (-p.lw / 2) + B * (-p.lh / 2),
    };
    V3 mn = c[0], mx = c[0];
    for (int i = 1; i < 4; ++i) {
        mn.x = mmin(mn.x, c[i].x); mn.y = mmin(mn.y, c[i].y); mn.z = mmin(mn.z, c[i].z);
        mx.x = mmax(mx.x, c[i].x); mx.y = mmax(mx.y, c[i].y); mx.z = mmax(mx.z, c[i].z);
    }
    p.box = pad(boxOf(mn, mx));
    return p;
}

static Prim makeSphere(const cpt_sphere& S, const Material& m)   // Hittable(Sphere) Hittable.cuh:418-422
{
    Prim p;
    p.kind = K_SPHERE;
    p.sc = v3(S.center[0], S.center[1], S.center[2]);
    p.r = S.radius;
    p.mat = m;
    p.center = p.sc;
    V3 rr = v3(p.r, p.r, p.r);
    p.box = boxOf(p.sc - rr, p.sc + rr);
    return p;
}

static Prim makeTriangle(V3 a, V3 b, V3 c, V3 na, V3 nb, V3 nc, const Material& m)   // Hittable.cuh:456-462
{
    Prim p;
    p.kind = K_TRI;
    p.p0 = a; p.p1 = b; p.p2 = c;
    p.n0 = na; p.n1 = nb; p.n2 = nc;
    for (double& x : p.uv) x = 0.0;
    p.tex = nullptr;
    p.texW = p.texH = 0;
    p.mat = m;
    p.center = (a + b + c) / 3.0;
    p.box = pad(boxOf(v3(mmin(mmin(a.x, b.x), c.x), mmin(mmin(a.y, b.y), c.y), mmin(mmin(a.z, b.z), c.z)),
                      v3(mmax(mmax(a.x, b.x), c.x), mmax(mmax(a.y, b.y), c.y), mmax(mmax(a.z, b.z), c.z))));
    return p;
}

// ------------------------------------------------------------------ intersection
static bool hitSphere(const Prim& p, const Ray& ray, HitRecord& rec, double tmin, double tmax)   // Hittable.cuh:27-54
{
    double a = dot(ray.d, ray.d);
    double b = dot(ray.d, ray.o - p.sc);
    double c = dot(ray.o - p.sc, ray.o - p.sc) - p.r * p.r;
    double delta = b * b - a * c;
    if (delta < 0.0) return false;
    double t = (-b - std::sqrt(delta)) / a;
    if (t < tmin || t > tmax) t = (-b + std::sqrt(delta)) / a;
    if (t < tmin || t > tmax) return false;
    rec.hitColor = p.mat.color;
    rec.hitPos = at(ray, t);
    rec.t = t;
    rec.material = &p.mat;
    V3 outward = (rec.hitPos - p.sc) / p.r;
    setFaceNormal(rec, ray, outward);
    return true;
}

static bool hitTriangle(const Prim& p, const Ray& ray, HitRecord& rec, double tmin, double tmax,
                        double* ou = nullptr, double* ov = nullptr)   // Hittable.cuh:85-140
{
    const double EPS = 1e-8;
    V3 e1 = p.p1 - p.p0;
    V3 e2 = p.p2 - p.p0;
    V3 h = cross(ray.d, e2);
    double a = dot(e1, h);
    if (std::fabs(a) < EPS) return false;
    double f = 1.0 / a;
    V3 s = ray.o - p.p0;
    double u = f * dot(s, h);
    if (u < 0.0 || u > 1.0) return false;
    V3 q = cross(s, e1);
    double v = f * dot(ray.d, q);
    if (v < 0.0 || u + v > 1.0) return false;
    double t = f * dot(e2, q);
    if (t < tmin || t > tmax) return false;
    if (p.tex) {   // Hittable.cuh:123-125
        double uu = (1.0 - u - v) * p.uv[0] + u * p.uv[2] + v * p.uv[4];
        double vv = (1.0 - u - v) * p.uv[1] + u * p.uv[3] + v * p.uv[5];
        rec.hitColor = texel(p.tex, p.texW, p.texH, uu, vv);
    } else {
        rec.hitColor = p.mat.color;   // sampleTexture(color) (HitRecord.cuh:34-37)
    }
    rec.hitPos = at(ray, t);
    rec.t = t;
    rec.material = &p.mat;
    if (p.n0.x < EPS && p.n0.y < EPS && p.n0.z < EPS && p.n1.x < EPS && p.n1.y < EPS && p.n1.z < EPS &&
        p.n2.x < EPS && p.n2.y < EPS && p.n2.z < EPS) {
        setFaceNormal(rec, ray, unit(cross(e1, e2)));
    } else {
        double w = 1.0 - u - v;
        setFaceNormal(rec, ray, unit(w * p.n0 + u * p.n1 + v * p.n2));
    }
    if (ou) *ou = u;
    if (ov) *ov = v;
    return true;
}

static bool hitLight(const Prim& p, const Ray& ray, HitRecord& rec, double tmin, double tmax)   // Hittable.cuh:367-398
{
    if (!p.visible) return false;
    double denom = dot(ray.d, p.ln);
    if (std::fabs(denom) < 1e-6 || denom > 0.0) return false;
    double t = dot(p.sc - ray.o, p.ln) / denom;
    if (t < tmin || t > tmax) return false;
    V3 hp = at(ray, t);
    V3 diff = hp - p.sc;
    double u = dot(diff, p.eu);
    double v = dot(diff, p.ev);
    if (std::fabs(u) <= p.lw / 2.0 && std::fabs(v) <= p.lh / 2.0) {
        rec.hitColor = p.mat.color;
        rec.hitPos = hp;
        rec.t = t;
        rec.material = &p.mat;
        setFaceNormal(rec, ray, p.ln);
        return true;
    }
    return false;
}

static bool hitPrim(const Prim& p, const Ray& ray, HitRecord& rec, double tmin, double tmax,
                    double* ou = nullptr, double* ov = nullptr)   // Hittable.cuh:487-503
{
    switch (p.kind) {
    case K_SPHERE: return hitSphere(p, ray, rec, tmin, tmax);
    case K_LIGHT: return hitLight(p, ray, rec, tmin, tmax);
    case K_TRI: return hitTriangle(p, ray, rec, tmin, tmax, ou, ov);
    }
    return false;
}

// ------------------------------------------------------------------ LBVH
static inline uint32_t expandBits(uint32_t v)   // BVH.cuh:12-19
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

static inline uint64_t morton3D(V3 c, V3 smin, V3 smax, int index)   // BVH.cuh:23-41
{
    double nx = (c.x - smin.x) / (smax.x - smin.x);
    double ny = (c.y - smin.y) / (smax.y - smin.y);
    double nz = (c.z - smin.z) / (smax.z - smin.z);
    double x = mmin(mmax(nx * 1024.0, 0.0), 1023.0);
    double y = mmin(mmax(ny * 1024.0, 0.0), 1023.0);
    double z = mmin(mmax(nz * 1024.0, 0.0), 1023.0);
    uint32_t xx = expandBits((uint32_t)x);
    uint32_t yy = expandBits((uint32_t)y);
    uint32_t zz = expandBits((uint32_t)z);
    uint64_t code = xx * 4 + yy * 2 + zz;
    return (code << 32) | (uint64_t)(int64_t)index;
}

static inline int clz64(uint64_t x) { return x == 0 ? 64 : __builtin_clzll(x); }

static int findSplit(const uint64_t* k, int first, int last)   // BVH.cuh:81-118
{
    uint64_t fc = k[first], lc = k[last];
    if (fc == lc) return (first + last) >> 1;
    int common = clz64(fc ^ lc);
    int split = first;
    int step = last - first;
    do {
        step = (step + 1) >> 1;
        int ns = split + step;
        if (ns < last) {
            if (clz64(fc ^ k[ns]) > common) split = ns;
        }
    } while (step > 1);
    return split;
}

static inline int delta(const uint64_t* k, int n, int i, int j)   // BVH.cuh:120-128
{
    if (j < 0 || j >= n) return -1;
    if (k[i] == k[j]) return 64;
    return clz64(k[i] ^ k[j]);
}

static void determineRange(const uint64_t* k, int n, int idx, int& first, int& last)   // BVH.cuh:130-172
{
    int dn = delta(k, n, idx, idx + 1);
    int dp = delta(k, n, idx, idx - 1);
    int d = (dn > dp) ? 1 : -1;
    int dmin = delta(k, n, idx, idx - d);
    int lmax = 2;
    while (delta(k, n, idx, idx + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta(k, n, idx, idx + (l + t) * d) > dmin) l += t;
    int j = idx + l * d;
    first = std::min(idx, j);
    last = std::max(idx, j);
}

struct Scene {
    std::vector<Prim> prims;
    int nLights = 0, nSpheres = 0, nTris = 0;
    // camera (Camera.cu:5-40)
    int width = 0, height = 0;
    V3 lookFrom, lookAt, background, dh, dv, pixelCenter;
    const uint8_t* sky = nullptr;   // equirectangular sky image (Camera::d_image) or NULL
    int skyW = 0, skyH = 0;
    V3 bmin, bmax;
    bool refMode = true;   // which estimator the materials were prepared for
    // LBVH (child encoding: >= 0 internal node, < 0 leaf ~k)
    std::vector<uint64_t> keys;
    std::vector<uint32_t> order;
    std::vector<int32_t> childA, childB;
    std::vector<Box> nodeBox, leafBox;
    bool built = false;
};

static void buildLBVH(Scene& s)   // Device::buildBVH, Device.cuh:169-195
{
    int n = (int)s.prims.size();
    V3 one = v3(1.0, 1.0, 1.0);
    V3 smin = s.bmin - one, smax = s.bmax + one;
    if (smin.x > smax.x) { smin = v3(-20.0, -20.0, -20.0); smax = v3(20.0, 20.0, 20.0); }
    s.keys.resize(n);
    s.order.resize(n);
    std::vector<uint64_t> raw(n);
    for (int i = 0; i < n; ++i) raw[i] = morton3D(s.prims[i].center, smin, smax, i);   // generateMortonCodes :134-142
    // thrust::sort_by_key (:187-189): keys are unique (the index is in the low word), so any
    // correct sort gives this permutation.
    std::vector<uint32_t> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = (uint32_t)i;
    std::sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return raw[a] < raw[b]; });
    for (int i = 0; i < n; ++i) { s.keys[i] = raw[idx[i]]; s.order[i] = idx[i]; }
    s.leafBox.resize(n);
    for (int i = 0; i < n; ++i) s.leafBox[i] = s.prims[s.order[i]].box;
    int ni = n > 1 ? n - 1 : 0;
    s.childA.assign(ni, 0);
    s.childB.assign(ni, 0);
    s.nodeBox.resize(ni);
    for (int i = 0; i < ni; ++i) {   // generateHierarchy (BVH.cuh:174-241)
        int first, last;
        determineRange(s.keys.data(), n, i, first, last);
        int split = findSplit(s.keys.data(), first, last);
        s.childA[i] = (split == first) ? ~split : split;
        s.childB[i] = (split + 1 == last) ? ~(split + 1) : split + 1;
    }
    // constructAABB (BVH.cuh:243-280): post-order union of the two children.
    if (ni > 0) {
        std::vector<int> stack;
        std::vector<char> done(ni, 0);
        stack.push_back(0);
        while (!stack.empty()) {
            int nd = stack.back();
            int a = s.childA[nd], b = s.childB[nd];
            bool ra = a < 0 || done[a], rb = b < 0 || done[b];
            if (ra && rb) {
                const Box& ba = a < 0 ? s.leafBox[~a] : s.nodeBox[a];
                const Box& bb = b < 0 ? s.leafBox[~b] : s.nodeBox[b];
                s.nodeBox[nd] = boxUnion(ba, bb);
                done[nd] = 1;
                stack.pop_back();
            } else {
                if (!rb) stack.push_back(b);
                if (!ra) stack.push_back(a);
            }
        }
    }
    s.built = true;
}

// ------------------------------------------------------------------ traversal
static inline bool checkSlab(double o, double inv, double mn, double mx, double& t0m, double& t1m)   // BVH.cuh:54-65
{
    double t0 = (mn - o) * inv;
    double t1 = (mx - o) * inv;
    if (inv < 0.0) std::swap(t0, t1);
    t0m = std::fmax(t0, t0m);
    t1m = std::fmin(t1, t1m);
    return t1m > t0m;
}

static inline bool checkOverlap(const Ray& r, const Box& b, double tmin, double tmax)   // BVH.cuh:66-79
{
    V3 inv = v3(1.0 / r.d.x, 1.0 / r.d.y, 1.0 / r.d.z);
    return checkSlab(r.o.x, inv.x, b.mn.x, b.mx.x, tmin, tmax) && checkSlab(r.o.y, inv.y, b.mn.y, b.mx.y, tmin, tmax) &&
           checkSlab(r.o.z, inv.z, b.mn.z, b.mx.z, tmin, tmax);
}

// traverseIterative (BVH.cuh:282-332): depth-first, both children tested against the
// original [tMin, tMax] (no pruning), leaves tested with [0.001, closest so far]; on equal
// t the later-visited leaf wins.  Single-primitive scenes (where the reference indexes an
// empty internal-node array) test the one leaf directly.
struct VisitCounts { uint64_t rays, vInt, vLeaf; };
static int traverseCounting(const Scene& s, const Ray& ray, double tMin, double tMax, uint64_t& vInt, uint64_t& vLeaf);
static thread_local VisitCounts* g_visit = nullptr;   // set while a render measures visit counts

static int traverse(const Scene& s, const Ray& ray, HitRecord& rec, double tMax = INF, double tMin = 0.001,
                    double* ou = nullptr, double* ov = nullptr)
{
    if (g_visit) {
        g_visit->rays++;
        traverseCounting(s, ray, tMin, tMax, g_visit->vInt, g_visit->vLeaf);
    }
    int n = (int)s.prims.size();
    int hitId = -1;
    HitRecord tmp;
    double bu = 0, bv = 0, tu = 0, tv = 0;
    if (n == 0) return -1;
    if (n == 1) {
        if (checkOverlap(ray, s.leafBox[0], tMin, tMax) &&
            hitPrim(s.prims[s.order[0]], ray, tmp, 0.001, tMax, &tu, &tv)) {
            rec = tmp;
            hitId = (int)s.order[0];
            bu = tu; bv = tv;
        }
        if (ou) *ou = bu;
        if (ov) *ov = bv;
        return hitId;
    }
    int stack[512];
    int sp = 0;
    stack[sp++] = INT32_MIN;   // sentinel (the reference pushes NULL)
    int node = 0;
    do {
        int cl = s.childA[node], cr = s.childB[node];
        const Box& bl = cl < 0 ? s.leafBox[~cl] : s.nodeBox[cl];
        const Box& br = cr < 0 ? s.leafBox[~cr] : s.nodeBox[cr];
        bool oL = checkOverlap(ray, bl, tMin, tMax);
        bool oR = checkOverlap(ray, br, tMin, tMax);
        if (oL && cl < 0) {
            int pid = (int)s.order[~cl];
            if (hitPrim(s.prims[pid], ray, tmp, 0.001, hitId >= 0 ? rec.t : tMax, &tu, &tv)) {
                hitId = pid;
                rec = tmp;
                bu = tu; bv = tv;
            }
        }
        if (oR && cr < 0) {
            int pid = (int)s.order[~cr];
            if (hitPrim(s.prims[pid], ray, tmp, 0.001, hitId >= 0 ? rec.t : tMax, &tu, &tv)) {
                hitId = pid;
                rec = tmp;
                bu = tu; bv = tv;
            }
        }
        bool trL = oL && cl >= 0;
        bool trR = oR && cr >= 0;
        if (!trL && !trR) {
            node = stack[--sp];
        } else {
            node = trL ? cl : cr;
            if (trL && trR) {
                if (sp >= 512) return -2;   // the reference would overflow its stack
                stack[sp++] = cr;
            }
        }
    } while (node != INT32_MIN);
    if (ou) *ou = bu;
    if (ov) *ov = bv;
    return hitId;
}

// Ordered, tMax-pruned traversal of the same binary LBVH, counting internal-node visits
// and primitive tests.  These counts define the algorithmic bytes per ray of the
// traversal roofline; the hit it returns is the same closest hit up to exact ties.
static int traverseCounting(const Scene& s, const Ray& ray, double tMin, double tMax, uint64_t& vInt, uint64_t& vLeaf)
{
    int n = (int)s.prims.size();
    if (n < 2) { vLeaf += n; return -1; }
    HitRecord tmp;
    double best = tMax;
    int hitId = -1;
    int stack[512];
    int sp = 0;
    int node = 0;
    for (;;) {
        vInt++;
        int c[2] = {s.childA[node], s.childB[node]};
        double tn[2];
        bool ov[2];
        for (int k = 0; k < 2; ++k) {
            const Box& b = c[k] < 0 ? s.leafBox[~c[k]] : s.nodeBox[c[k]];
            V3 inv = v3(1.0 / ray.d.x, 1.0 / ray.d.y, 1.0 / ray.d.z);
            double t0 = tMin, t1 = best;
            ov[k] = checkSlab(ray.o.x, inv.x, b.mn.x, b.mx.x, t0, t1) && checkSlab(ray.o.y, inv.y, b.mn.y, b.mx.y, t0, t1) &&
                    checkSlab(ray.o.z, inv.z, b.mn.z, b.mx.z, t0, t1);
            tn[k] = t0;
        }
        int next = -1;
        int push = -1;
        for (int k = 0; k < 2; ++k) {
            if (!ov[k]) continue;
            if (c[k] < 0) {
                vLeaf++;
                int pid = (int)s.order[~c[k]];
                if (hitPrim(s.prims[pid], ray, tmp, 0.001, best)) { best = tmp.t; hitId = pid; }
            }
        }
        bool tl = ov[0] && c[0] >= 0, tr = ov[1] && c[1] >= 0;
        if (tl && tr) {
            bool leftNear = tn[0] <= tn[1];
            next = leftNear ? c[0] : c[1];
            push = leftNear ? c[1] : c[0];
        } else if (tl) {
            next = c[0];
        } else if (tr) {
            next = c[1];
        }
        if (push >= 0 && sp < 512) stack[sp++] = push;
        if (next >= 0) { node = next; continue; }
        if (sp == 0) break;
        node = stack[--sp];
    }
    return hitId;
}

// ------------------------------------------------------------------ BSDF (Material.cuh)
static V3 worldToLocal(V3 N, V3 W)   // Material.cuh:238-248
{
    V3 z = N;
    V3 up = v3(0.0, 0.0, 1.0);
    if (std::fabs(dot(z, up)) > 0.99999) up = v3(1.0, 0.0, 0.0);
    V3 x = unit(cross(up, z));
    V3 y = cross(z, x);
    return v3(dot(W, x), dot(W, y), dot(W, z));
}

static double ggxD(const Material& m, V3 N, V3 H)   // Material.cuh:250-265
{
    V3 w = worldToLocal(N, H);
    double sinT = std::sqrt(1.0 - w.z * w.z);
    double cosP = w.x / sinT;
    double sinP = w.y / sinT;
    double cos2 = w.z * w.z;
    double sin2 = 1.0 - cos2;
    double tan2 = sin2 / cos2;
    double cos4 = cos2 * cos2;
    double cDa = cosP / m.ax;
    double sDa = sinP / m.ay;
    double e = tan2 * (cDa * cDa + sDa * sDa);
    return 1.0 / (PI * m.ax * m.ay * cos4 * (1 + e) * (1 + e));
}

static double lambda(const Material& m, V3 N, V3 R)   // Material.cuh:266-277
{
    V3 w = worldToLocal(N, R);
    double sinT = std::sqrt(1 - w.z * w.z);
    double cosP = w.x / sinT;
    double sinP = w.y / sinT;
    double alpha2 = m.ax * m.ax * cosP * cosP + m.ay * m.ay * sinP * sinP;
    double alpha = std::sqrt(alpha2);
    double tanT = std::tan(std::acos(mmax(dot(N, R), 0.0)));
    return (std::sqrt(1.0 + alpha * alpha * tanT * tanT) - 1.0) / 2.0;
}

static double smithG2(const Material& m, V3 N, V3 V, V3 L) { return 1.0 / (1.0 + lambda(m, N, V) + lambda(m, N, L)); }   // :278-281
static double smithG1(const Material& m, V3 N, V3 W) { return 1.0 / (1.0 + lambda(m, N, W)); }                         // :282-285

static double fresnelConductor(V3 N, V3 V, V3 L, double n, double k)   // Material.cuh:287-295
{
    C2 eta = c2(n, k);
    double ci = mmax(dot(N, V), 0.0);
    double ct = mmax(dot(N, L), 0.0);
    C2 ec = c2(ci * eta.x, ci * eta.y);
    C2 rpar = cdiv(c2(ec.x - ct, ec.y), c2(ct + ec.x, ec.y));
    C2 et = c2(ct * eta.x, ct * eta.y);
    C2 rper = cdiv(c2(ci - et.x, -et.y), c2(ci + et.x, et.y));
    return (cnorm(rpar) + cnorm(rper)) / 2.0;
}

static double fresnelDielectric(V3 N, V3 V, double eta)   // Material.cuh:305-318
{
    double ci = std::fabs(dot(N, V));
    double si = std::sqrt(mmax(0.0, 1.0 - ci * ci));
    double st = si / eta;
    if (st >= 1.0) return 1.0;
    double ct = std::sqrt(mmax(0.0, 1.0 - st * st));
    double rpar = (eta * ci - ct) / (eta * ci + ct);
    double rper = (ci - eta * ct) / (ci + eta * ct);
    return (rpar * rpar + rper * rper) * 0.5;
}

static V3 bsdfEval(const Material& m, V3 hitColor, const Ray& ray, V3 normal, V3 dir, V3 wm, bool front)   // Material::fr :24-93
{
    if (m.type == M_LAMBERT) return hitColor / PI;
    V3 V = unit(-ray.d);
    V3 L = unit(dir);
    V3 H = unit(V + L);
    bool reflect = dot(V, normal) * dot(L, normal) > 0.0;
    if (m.type == M_SPEC) {
        double rr = front ? m.eta : (1.0 / m.eta);
        double ct = std::fabs(dot(normal, L));
        double F = fresnelDielectric(normal, V, rr);
        if (reflect) return F * hitColor / ct;
        return (1.0 - F) * hitColor / ct;
    } else if (!reflect) {
        double rr = front ? m.eta : (1.0 / m.eta);
        double D = ggxD(m, normal, wm);
        if (dot(wm, V) < 0.0) V = -V;
        if (dot(wm, L) < 0.0) L = -L;
        double G = smithG2(m, normal, V, L);
        double F = fresnelDielectric(wm, V, rr);
        double ci = std::fabs(dot(normal, V));
        double ct = std::fabs(dot(normal, L));
        double mb = std::fabs(dot(L, wm)) + std::fabs(dot(V, wm)) / rr;
        double den = mb * mb;
        double spec = (1.0 - F) * D * G * std::fabs(dot(wm, L) * dot(wm, V) / (ci * ct * den));
        return spec * hitColor;
    } else {
        double n = 2.63, k = 9.08;
        if (m.type == M_ROUGH) { n = 1.58; k = 0.001; }
        double D = ggxD(m, normal, H);
        double G = smithG2(m, normal, V, L);
        double F = fresnelConductor(normal, V, L, n, k);
        double NdotL = mmax(dot(normal, L), 0.0);
        double NdotV = mmax(dot(normal, V), 0.0);
        double den = 4.0 * NdotV * NdotL + 0.001;
        double spec = (D * G * F) / den;
        return spec * hitColor;
    }
}

static const double ONE_E_MINUS_6F = (double)1e-6f;   // mMax(1e-6f, nh.z), Material.cuh:140,222

static void sampleGGXReflect(const Material& m, const Ray& ray, V3 normal, V3& dir, double& pdf, double r1, double r2)   // brdf :201-235
{
    V3 w = normal;
    V3 a = (std::fabs(w.z) > 0.99999) ? v3(1.0, 0.0, 0.0) : v3(0.0, 0.0, 1.0);
    V3 u = unit(cross(a, w));
    V3 v = cross(w, u);
    V3 urd = -unit(ray.d);
    V3 Wo = v3(dot(urd, u), dot(urd, v), dot(urd, w));
    V3 Wh = unit(v3(m.ax * Wo.x, m.ay * Wo.y, Wo.z));
    V3 T1 = (Wh.z < 0.99999) ? unit(cross(v3(0, 0, 1), Wh)) : unit(cross(v3(1, 0, 0), Wh));
    V3 T2 = cross(Wh, T1);
    double r = std::sqrt(r1);
    double theta = 2 * PI * r2;
    double px = r * std::cos(theta), py = r * std::sin(theta);
    double h = std::sqrt(1 - px * px);
    double lx = (1 + Wh.z) / 2.0;
    py = (1.0 - lx) * h + lx * py;
    double pz = std::sqrt(mmax(0.0, 1.0 - (px * px + py * py)));
    V3 nh = px * T1 + py * T2 + pz * Wh;
    V3 Wm = unit(v3(m.ax * nh.x, m.ay * nh.y, mmax(ONE_E_MINUS_6F, nh.z)));
    V3 Wi = -Wo + 2 * dot(Wo, Wm) * Wm;
    dir = unit(Wi.x * u + Wi.y * v + Wi.z * w);
    if (dot(dir, normal) < 0.0) { pdf = -1.0; return; }
    V3 H = unit(dir + urd);
    pdf = smithG1(m, normal, urd) / Wo.z * ggxD(m, normal, H) / 4.0;
}

static void bsdfSample(const Material& m, const Ray& ray, V3 normal, V3& dir, V3& wm, double& pdf, double r1, double r2,
                       double r3, bool front)   // Material::sampleLight :95-193
{
    if (m.type == M_SPEC) {
        double rr = front ? m.eta : (1.0 / m.eta);
        V3 urd = unit(ray.d);
        double R = fresnelDielectric(normal, -urd, rr);
        if (r3 < R) {
            dir = urd - 2.0 * dot(urd, normal) * normal;
            pdf = R;
        } else {
            V3 vperp = 1.0 / rr * (urd + dot(-urd, normal) * normal);
            V3 vpar = -std::sqrt(std::fabs(1.0 - len2(vperp))) * normal;
            dir = unit(vperp + vpar);
            pdf = 1.0 - R;
        }
    } else if (m.type == M_ROUGH) {
        V3 w = normal;
        V3 a = (std::fabs(w.x) > 0.9) ? v3(0.0, 1.0, 0.0) : v3(1.0, 0.0, 0.0);
        V3 u = unit(cross(w, a));
        V3 v = cross(w, u);
        V3 urd = -unit(ray.d);
        V3 Wo = v3(dot(urd, u), dot(urd, v), dot(urd, w));
        V3 Wh = unit(v3(m.ax * Wo.x, m.ay * Wo.y, Wo.z));
        V3 T1 = (Wh.z < 0.99999) ? unit(cross(v3(0, 0, 1), Wh)) : v3(1, 0, 0);
        V3 T2 = cross(Wh, T1);
        double r = std::sqrt(r1);
        double theta = 2 * PI * r2;
        double px = r * std::cos(theta), py = r * std::sin(theta);
        double h = std::sqrt(1 - px * px);
        double lx = (1 + Wh.z) / 2.0;
        py = (1.0 - lx) * h + lx * py;
        double pz = std::sqrt(mmax(0.0, 1.0 - (px * px + py * py)));
        V3 nh = px * T1 + py * T2 + pz * Wh;
        V3 Wm = unit(v3(m.ax * nh.x, m.ay * nh.y, mmax(ONE_E_MINUS_6F, nh.z)));
        V3 sn = unit(Wm.x * u + Wm.y * v + Wm.z * w);
        wm = sn;
        double rr = front ? m.eta : (1.0 / m.eta);
        double R = fresnelDielectric(sn, -urd, rr);
        if (r3 < R) {
            sampleGGXReflect(m, ray, normal, dir, pdf, r1, r2);
            pdf *= R;
        } else {
            V3 vperp = 1.0 / rr * (urd + dot(-urd, sn) * sn);
            V3 vpar = -std::sqrt(std::fabs(1.0 - len2(vperp))) * sn;
            V3 rd = unit(vperp + vpar);
            V3 Wi = v3(dot(rd, u), dot(rd, v), dot(rd, w));
            dir = rd;
            if (dot(dir, normal) > 0.0) { pdf = -1.0; return; }
            double mb = dot(-Wi, Wm) + dot(Wo, Wm) / rr;
            double den = mb * mb;
            double dwm = std::fabs(dot(Wi, Wm)) / den;
            pdf = smithG1(m, normal, urd) / Wo.z * ggxD(m, normal, sn) * dot(Wo, Wm) * dwm * (1.0 - R);
        }
    } else if (m.type == M_OPAQUE) {
        sampleGGXReflect(m, ray, normal, dir, pdf, r1, r2);
    } else if (m.type == M_LAMBERT) {
        // Cosine-weighted hemisphere (the reference's commented-out sampler, Material.cuh:177-188).
        double sinT = std::sqrt(1.0 - r1);
        double cosT = std::sqrt(r1);
        V3 w = normal;
        V3 a = (std::fabs(w.x) > 0.9) ? v3(0.0, 1.0, 0.0) : v3(1.0, 0.0, 0.0);
        V3 u = unit(cross(w, a));
        V3 v = cross(w, u);
        dir = std::cos(2.0 * PI * r2) * sinT * u + std::sin(2.0 * PI * r2) * sinT * v + cosT * w;
        pdf = cosT / PI;
    }
}

// ------------------------------------------------------------------ camera (Camera.cu:5-40)
static void setupCamera(Scene& s, const cpt_camera& c)
{
    s.width = c.width;
    double aspect = c.aspect_ratio;
    s.height = c.width / aspect < 1 ? 1 : (int)(c.width / aspect);
    s.lookFrom = v3(c.look_from[0], c.look_from[1], c.look_from[2]);
    s.lookAt = v3(c.look_at[0], c.look_at[1], c.look_at[2]);
    s.background = v3(c.background[0], c.background[1], c.background[2]);
    V3 vUp = v3(0, 1, 0);
    double focal = length(s.lookFrom - s.lookAt);
    double theta = c.vfov_deg * PI / 180.0;
    double h = std::tan(theta / 2);
    double vh = 2.0 * h * focal;
    double vw = (double)s.width / s.height * vh;
    V3 w = unit(s.lookFrom - s.lookAt);
    V3 u = unit(cross(vUp, w));
    V3 v = cross(w, u);
    V3 hor = vw * u;
    V3 ver = vh * v;
    s.dh = hor / s.width;
    s.dv = ver / s.height;
    V3 ul = s.lookFrom - hor / 2 - ver / 2 - focal * w;
    s.pixelCenter = ul + s.dh / 2 + s.dv / 2;
}

static V3 skyBox(const Scene& s, V3 direction)   // Camera::getSkyBox, Camera.cuh:50-63
{
    if (!s.sky) return s.background;
    V3 dir = unit(direction);
    double u = std::atan2(-dir.z, dir.x) / (2.0 * PI) + 0.5;
    double v = 0.5 - std::asin(dir.y) / PI;
    return texel(s.sky, s.skyW, s.skyH, u, v);
}

static inline Ray cameraRay(const Scene& s, int x, int y, double rx, double ry)   // Camera.cuh:37-43
{
    V3 p = s.pixelCenter + (rx - 0.5 + x) * s.dh + (ry - 0.5 + y) * s.dv;
    Ray r = {s.lookFrom, p - s.lookFrom};
    return r;
}

// ------------------------------------------------------------------ render
struct PixelOut {
    V3 rgb;
    V3 gN; double gDepth; V3 gAlbedo;
    double gVar;   // config estimator: variance of the pixel mean's luminance
    uint64_t rays;
};

static inline double luminance(V3 c) { return 0.2126 * c.x + 0.7152 * c.y + 0.0722 * c.z; }

// The reference's STATIC render for one pixel (Render.cu:20-227).
static PixelOut renderPixelReference(const Scene& s, int i, int j, int spp, uint64_t seed)
{
    PixelOut out = {};
    int offset = j * s.width + i;
    Rng st;
    st.init(seed, (uint64_t)offset);
    V3 pix = v3(0, 0, 0);
    uint64_t rays = 0;
    for (int sample = 0; sample < spp; ++sample) {
        double rx = st.uniform();
        double ry = st.uniform();
        Ray ray = cameraRay(s, i, j, rx, ry);
        V3 thr = v3(1.0, 1.0, 1.0);
        V3 rad = v3(0.0, 0.0, 0.0);
        out.gN = v3(0, 0, 0); out.gDepth = INF; out.gAlbedo = v3(0, 0, 0); out.gVar = 0.0;
        bool hasSampleLight = false;
        for (;;) {
            HitRecord rec;
            HitRecord lrec;
            int hitId = traverse(s, ray, rec);
            rays++;
            if (hitId >= 0 && rec.material->type == M_VOLUME) {   // :64-135
                double sig = 25.0;
                HitRecord vrec;
                ray.o = rec.hitPos;
                int isHit = traverse(s, ray, vrec);
                rays++;
                if (isHit < 0) continue;
                double dMax = vrec.t;
                double t = -std::log(1.0 - st.uniform()) / sig;
                V3 pos = rec.hitPos + t * ray.d;
                ray.o = pos;
                while (t < dMax) {
                    double P = 0.8;
                    if (st.uniform() > P) break;
                    thr = thr * (std::exp(-t * sig) / P);
                    double z = 1.0 - 2.0 * st.uniform();
                    double r = std::sqrt(1.0 - z * z);
                    double phi = 2.0 * PI * st.uniform();
                    V3 d = unit(v3(r * std::cos(phi), r * std::sin(phi), z));
                    ray.o = pos;
                    ray.d = d;
                    pos = rec.hitPos + t * d;
                    isHit = traverse(s, ray, vrec);
                    rays++;
                    dMax = vrec.t;
                    t = -std::log(1.0 - st.uniform()) / sig;
                    if (t > dMax || isHit < 0) break;
                }
                continue;
            }
            if (hitId < 0) { rad = rad + thr * skyBox(s, ray.d); break; }
            if (rec.material->type == M_LIGHT) {
                if (!hasSampleLight) rad = rad + thr * rec.hitColor;
                break;
            }
            // G-buffer: the reference's depth stays 0 in STATIC mode, so the last surface wins (:152-159).
            out.gN = rec.normal;
            out.gDepth = length(s.lookFrom - rec.hitPos);
            out.gAlbedo = rec.hitColor;
            V3 dir;
            for (int k = 0; k < s.nLights; ++k) {   // :163-187
                if (rec.material->type != M_OPAQUE) break;
                const Prim& L = s.prims[k];
                double lw = L.lw;
                double lh = L.lw;   // the reference uses the width for both sides (:171)
                double pdfL = 1.0 / (lw * lh);
                // g++ evaluates the second draw of this expression first (the C++ order of
                // the two operands is unspecified); the oracle follows the compiled reference.
                double ub = st.uniform();
                double ua = st.uniform();
                V3 lp = L.sc + (ua - 0.5) * lw * L.eu + (ub - 0.5) * lh * L.ev;
                dir = unit(lp - rec.hitPos);
                Ray sr = {rec.hitPos, dir};
                int obst = traverse(s, sr, lrec);
                rays++;
                if (dot(dir, rec.normal) > 0.0 && dot(-dir, L.ln) > 0.0 && obst == k) {
                    V3 fr = bsdfEval(*rec.material, rec.hitColor, ray, rec.normal, dir, rec.hitWm, rec.frontFace);
                    V3 cl = lrec.hitColor * fr * dot(dir, rec.normal) * dot(-dir, L.ln) / len2(lp - rec.hitPos) / pdfL;
                    rad = rad + thr * cl;
                }
                hasSampleLight = true;
            }
            double P = 0.7;   // STATIC: Russian roulette every bounce (:199-204)
            if (st.uniform() > P) break;
            double r1 = st.uniform(), r2 = st.uniform(), r3 = st.uniform();
            double pdf;
            bsdfSample(*rec.material, ray, rec.normal, dir, rec.hitWm, pdf, r1, r2, r3, rec.frontFace);
            if (pdf <= 0.0) break;
            V3 fr = bsdfEval(*rec.material, rec.hitColor, ray, rec.normal, dir, rec.hitWm, rec.frontFace);
            thr = thr * (fr * std::fabs(dot(dir, rec.normal)) / pdf / P);
            ray.o = rec.hitPos;
            ray.d = dir;
        }
        pix = pix + rad;
    }
    pix = v3(pix.x / spp, pix.y / spp, pix.z / spp);
    out.rgb = pix;
    out.rays = rays;
    return out;
}

// The config estimator (no reference code): depth limit, RR from rr_depth on, NEE at
// Opaque and Lambertian vertices with the true light area, emission counted only when the
// previous vertex did not sample the lights, homogeneous media bounded by CPT_M_VOLUME
// surfaces (free-flight sampling with sigma_t, throughput *= albedo per scattering).
static PixelOut renderPixelConfig(const Scene& s, int i, int j, const cpt_render_params& p)
{
    PixelOut out = {};
    int offset = j * s.width + i;
    const int group = sampleGroup(p.spp);
    V3 pix = v3(0, 0, 0), gsum = v3(0, 0, 0);
    double sumY2 = 0.0;
    uint64_t rays = 0;
    out.gDepth = INF;
    for (int sample = 0; sample < p.spp; ++sample) {
        Rng st;
        st.init(p.seed, (uint64_t)offset);
        st.advance((uint64_t)sample << 32);
        double rx = st.uniform();
        double ry = st.uniform();
        Ray ray = cameraRay(s, i, j, rx, ry);
        V3 thr = v3(1.0, 1.0, 1.0);
        V3 rad = v3(0.0, 0.0, 0.0);
        bool countEmission = true;
        bool inMedium = false;
        double mSigma = 0.0, mAlbedo = 0.0;
        int depth = 0;
        int guard = 0;
        for (;;) {
            if (++guard > 100000) break;
            HitRecord rec;
            int hitId = traverse(s, ray, rec);
            rays++;
            if (inMedium) {
                double tHit = hitId >= 0 ? rec.t : INF;
                double t = -std::log(st.uniform()) / mSigma;
                if (t < tHit) {
                    V3 pos = at(ray, t);
                    thr = thr * mAlbedo;
                    depth++;
                    if (p.max_depth > 0 && depth >= p.max_depth) break;
                    double P = 1.0;
                    if (depth >= p.rr_depth) {
                        P = p.rr_prob;
                        if (st.uniform() > P) break;
                    }
                    thr = thr * (1.0 / P);
                    double z = 1.0 - 2.0 * st.uniform();
                    double r = std::sqrt(mmax(0.0, 1.0 - z * z));
                    double phi = 2.0 * PI * st.uniform();
                    ray.o = pos;
                    ray.d = v3(r * std::cos(phi), r * std::sin(phi), z);
                    countEmission = true;
                    continue;
                }
            }
            if (hitId < 0) { rad = rad + thr * skyBox(s, ray.d); break; }
            const Material& m = *rec.material;
            if (m.type == M_VOLUME) {
                inMedium = rec.frontFace;
                mSigma = m.sigma_t;
                mAlbedo = m.albedo;
                ray.o = rec.hitPos;
                continue;
            }
            if (m.type == M_LIGHT) {
                if (countEmission) rad = rad + thr * rec.hitColor;
                break;
            }
            if (depth == 0 && sample < group && out.gDepth >= INF) {
                out.gN = rec.normal;
                out.gDepth = length(s.lookFrom - rec.hitPos);
                out.gAlbedo = rec.hitColor;
            }
            bool diffuseLike = (m.type == M_OPAQUE || m.type == M_LAMBERT);
            if (diffuseLike) {
                for (int k = 0; k < s.nLights; ++k) {
                    const Prim& L = s.prims[k];
                    double area = L.lw * L.lh;
                    double ua = st.uniform();
                    double ub = st.uniform();
                    V3 lp = L.sc + (ua - 0.5) * L.lw * L.eu + (ub - 0.5) * L.lh * L.ev;
                    V3 dir = unit(lp - rec.hitPos);
                    double cs = dot(dir, rec.normal), cl = dot(-dir, L.ln);
                    if (!(cs > 0.0 && cl > 0.0)) continue;   // cannot contribute: no shadow ray
                    Ray sr = {rec.hitPos, dir};
                    HitRecord lrec;
                    // a ray that misses the light itself (an invisible light) cannot see it: not traced
                    if (!hitLight(L, sr, lrec, 0.001, INF)) continue;
                    int obst = traverse(s, sr, lrec);
                    rays++;
                    if (obst == k) {
                        V3 fr = bsdfEval(m, rec.hitColor, ray, rec.normal, dir, rec.hitWm, rec.frontFace);
                        double g = cs * cl / len2(lp - rec.hitPos) * area;
                        rad = rad + thr * (lrec.hitColor * fr * g);
                    }
                }
            }
            countEmission = !diffuseLike || s.nLights == 0;
            depth++;
            if (p.max_depth > 0 && depth >= p.max_depth) break;
            double P = 1.0;
            if (depth >= p.rr_depth) {
                P = p.rr_prob;
                if (st.uniform() > P) break;
            }
            double r1 = st.uniform(), r2 = st.uniform(), r3 = st.uniform();
            double pdf;
            V3 dir;
            bsdfSample(m, ray, rec.normal, dir, rec.hitWm, pdf, r1, r2, r3, rec.frontFace);
            if (pdf <= 0.0) break;
            V3 fr = bsdfEval(m, rec.hitColor, ray, rec.normal, dir, rec.hitWm, rec.frontFace);
            thr = thr * (fr * std::fabs(dot(dir, rec.normal)) / pdf / P);
            ray.o = rec.hitPos;
            ray.d = dir;
        }
        gsum = gsum + rad;
        sumY2 += luminance(rad) * luminance(rad);
        if ((sample + 1) % group == 0 || sample + 1 == p.spp) {
            pix = pix + gsum;
            gsum = v3(0, 0, 0);
        }
    }
    // the sample variance of the luminance over the samples, divided by spp (one sample: Y^2)
    const double ys = luminance(pix);
    out.gVar = p.spp <= 1 ? sumY2 : std::max(0.0, (sumY2 - ys * ys / p.spp) / ((double)(p.spp - 1) * p.spp));
    pix = v3(pix.x / p.spp, pix.y / p.spp, pix.z / p.spp);
    out.rgb = pix;
    out.rays = rays;
    return out;
}

static Material toMaterial(const cpt_material& m, bool refMode)
{
    Material r;
    r.color = v3(m.color[0], m.color[1], m.color[2]);
    r.ax = m.alpha_x;
    r.ay = m.alpha_y;
    r.type = m.type;
    r.eta = refMode ? 1.51 : m.eta;
    r.sigma_t = m.sigma_t;
    r.albedo = m.albedo;
    if (refMode && (r.type == M_LAMBERT || r.type < M_LIGHT || r.type > M_VOLUME)) r.type = M_OPAQUE;
    return r;
}

static int buildScene(Scene& s, const cpt_scene_desc* d, bool refMode)
{
    s.prims.clear();
    s.refMode = refMode;
    s.nLights = (int)d->num_lights;
    s.nSpheres = (int)d->num_spheres;
    s.nTris = (int)d->num_triangles;
    for (uint32_t i = 0; i < d->num_lights; ++i) s.prims.push_back(makeLight(d->lights[i]));
    for (uint32_t i = 0; i < d->num_spheres; ++i) {
        uint32_t mi = d->spheres[i].material;
        if (mi >= d->num_materials) return 1;
        s.prims.push_back(makeSphere(d->spheres[i], toMaterial(d->materials[mi], refMode)));
    }
    for (uint32_t i = 0; i < d->num_triangles; ++i) {
        V3 p[3], n[3];
        for (int k = 0; k < 3; ++k) {
            if (d->tri_vertices_f64)
                p[k] = v3(d->tri_vertices_f64[9 * i + 3 * k], d->tri_vertices_f64[9 * i + 3 * k + 1],
                          d->tri_vertices_f64[9 * i + 3 * k + 2]);
            else
                p[k] = v3(d->tri_vertices[9 * i + 3 * k], d->tri_vertices[9 * i + 3 * k + 1], d->tri_vertices[9 * i + 3 * k + 2]);
            if (d->tri_normals)
                n[k] = v3(d->tri_normals[9 * i + 3 * k], d->tri_normals[9 * i + 3 * k + 1], d->tri_normals[9 * i + 3 * k + 2]);
            else
                n[k] = v3(0, 0, 0);
        }
        uint32_t mi = d->tri_material ? d->tri_material[i] : 0;
        if (mi >= d->num_materials) return 1;
        s.prims.push_back(makeTriangle(p[0], p[1], p[2], n[0], n[1], n[2], toMaterial(d->materials[mi], refMode)));
        Prim& t = s.prims.back();
        if (d->tri_uvs)
            for (int k = 0; k < 6; ++k) t.uv[k] = d->tri_uvs[6 * i + k];
        int tx = d->materials[mi].texture;
        if (tx < 0 || (uint32_t)tx > d->num_textures) return 1;
        if (tx > 0) {
            const cpt_image& im = d->textures[tx - 1];
            t.tex = im.rgb;
            t.texW = im.width;
            t.texH = im.height;
        }
    }
    if (d->sky.rgb) {
        s.sky = d->sky.rgb;
        s.skyW = d->sky.width;
        s.skyH = d->sky.height;
    }
    s.bmin = v3(d->bounds_min[0], d->bounds_min[1], d->bounds_min[2]);
    s.bmax = v3(d->bounds_max[0], d->bounds_max[1], d->bounds_max[2]);
    setupCamera(s, d->camera);
    return 0;
}

struct Handle {
    Scene ref;      // materials as the reference estimator sees them
    Scene cfg;      // materials for the config estimator (shares geometry and BVH)
};

static void parallelRows(int r0, int r1, int threads, const std::function<void(int)>& fn)
{
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<int> next(r0);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&]() {
            for (;;) {
                int r = next.fetch_add(1);
                if (r >= r1) break;
                fn(r);
            }
        });
    for (auto& th : pool) th.join();
}
}  // namespace orc

using namespace orc;

ORC_API void* orc_scene_create(const cpt_scene_desc* d)
{
    Handle* h = new Handle();
    if (buildScene(h->ref, d, true) || buildScene(h->cfg, d, false)) { delete h; return nullptr; }
    buildLBVH(h->ref);
    // Geometry (and therefore the LBVH) is identical under both estimators.
    h->cfg.keys = h->ref.keys; h->cfg.order = h->ref.order; h->cfg.childA = h->ref.childA;
    h->cfg.childB = h->ref.childB; h->cfg.nodeBox = h->ref.nodeBox; h->cfg.leafBox = h->ref.leafBox;
    h->cfg.built = true;
    return h;
}

ORC_API void orc_scene_destroy(void* p) { delete (Handle*)p; }

ORC_API int orc_scene_size(void* p, int* w, int* hgt)
{
    Handle* h = (Handle*)p;
    if (w) *w = h->ref.width;
    if (hgt) *hgt = h->ref.height;
    return (int)h->ref.prims.size();
}

// Binary LBVH in the C-ABI's export layout (boxes in FP64).
ORC_API int orc_lbvh_export(void* p, uint64_t* keys, uint32_t* order, int32_t* ca, int32_t* cb, double* nodeBoxes,
                            double* leafBoxes, double* centroids)
{
    const Scene& s = ((Handle*)p)->ref;
    int n = (int)s.prims.size();
    for (int i = 0; i < n; ++i) {
        if (keys) keys[i] = s.keys[i];
        if (order) order[i] = s.order[i];
        if (leafBoxes) {
            const Box& b = s.leafBox[i];
            double v[6] = {b.mn.x, b.mn.y, b.mn.z, b.mx.x, b.mx.y, b.mx.z};
            std::memcpy(leafBoxes + 6 * i, v, sizeof v);
        }
        if (centroids) {
            centroids[3 * i] = s.prims[i].center.x;
            centroids[3 * i + 1] = s.prims[i].center.y;
            centroids[3 * i + 2] = s.prims[i].center.z;
        }
    }
    for (int i = 0; i + 1 < n; ++i) {
        if (ca) ca[i] = s.childA[i];
        if (cb) cb[i] = s.childB[i];
        if (nodeBoxes) {
            const Box& b = s.nodeBox[i];
            double v[6] = {b.mn.x, b.mn.y, b.mn.z, b.mx.x, b.mx.y, b.mx.z};
            std::memcpy(nodeBoxes + 6 * i, v, sizeof v);
        }
    }
    return n;
}

// Closest hit per ray with the reference's traversal; rays are 8 doubles (o, tmin, d, tmax).
// out_id[i] = primitive index or -1, out_t/out_u/out_v the hit parameters.
ORC_API void orc_trace(void* p, const double* rays, int64_t n, int32_t* outId, double* outT, double* outU, double* outV,
                       int threads)
{
    const Scene& s = ((Handle*)p)->ref;
    const int64_t chunk = 1024;
    int nchunks = (int)((n + chunk - 1) / chunk);
    parallelRows(0, nchunks, threads, [&](int c) {
        for (int64_t i = c * chunk; i < std::min(n, (int64_t)(c + 1) * chunk); ++i) {
            const double* r = rays + 8 * i;
            Ray ray = {v3(r[0], r[1], r[2]), v3(r[4], r[5], r[6])};
            HitRecord rec;
            double u = 0, v = 0;
            int id = traverse(s, ray, rec, r[7], r[3], &u, &v);
            outId[i] = id;
            if (outT) outT[i] = id >= 0 ? rec.t : -1.0;
            if (outU) outU[i] = u;
            if (outV) outV[i] = v;
        }
    });
}

// Exact t of ray i against primitive prim (no BVH); -1 when it misses.  Used to classify
// near-tie disagreements.
ORC_API void orc_prim_t(void* p, const double* rays, int64_t n, const int32_t* prims, double* outT)
{
    const Scene& s = ((Handle*)p)->ref;
    for (int64_t i = 0; i < n; ++i) {
        const double* r = rays + 8 * i;
        Ray ray = {v3(r[0], r[1], r[2]), v3(r[4], r[5], r[6])};
        HitRecord rec;
        int pid = prims[i];
        outT[i] = (pid >= 0 && pid < (int)s.prims.size() && hitPrim(s.prims[pid], ray, rec, 0.001, r[7])) ? rec.t : -1.0;
    }
}

// Visit counts of the ordered, pruned traversal (internal nodes, primitive tests).
ORC_API void orc_trace_counts(void* p, const double* rays, int64_t n, uint64_t* vInt, uint64_t* vLeaf, int threads)
{
    const Scene& s = ((Handle*)p)->ref;
    std::atomic<uint64_t> ai(0), al(0);
    const int64_t chunk = 1024;
    int nchunks = (int)((n + chunk - 1) / chunk);
    parallelRows(0, nchunks, threads, [&](int c) {
        uint64_t li = 0, ll = 0;
        for (int64_t i = c * chunk; i < std::min(n, (int64_t)(c + 1) * chunk); ++i) {
            const double* r = rays + 8 * i;
            Ray ray = {v3(r[0], r[1], r[2]), v3(r[4], r[5], r[6])};
            traverseCounting(s, ray, r[3], r[7], li, ll);
        }
        ai += li;
        al += ll;
    });
    *vInt = ai.load();
    *vLeaf = al.load();
}

// Renders rows [p->row_begin, p->row_end) (all rows when both are 0).  rgb is W*H*3 doubles;
// rgba8 (optional) W*H*4 bytes with the reference's display encoding (Render.cu:229-260);
// gbuf (optional) W*H*8 doubles.  Returns the number of closest-hit queries traced.
ORC_API uint64_t orc_render(void* p, const cpt_render_params* prm, double* rgb, uint8_t* rgba8, double* gbuf, int threads)
{
    Handle* h = (Handle*)p;
    bool ref = prm->estimator == CPT_ESTIMATOR_REFERENCE;
    const Scene& s = ref ? h->ref : h->cfg;
    int r0 = prm->row_begin, r1 = prm->row_end;
    if (r0 == 0 && r1 == 0) r1 = s.height;
    std::atomic<uint64_t> total(0);
    // pixels of the band in chunks of 16, so that a band of few rows still uses every thread
    const int64_t npix = (int64_t)(r1 > r0 ? r1 - r0 : 0) * s.width;
    const int chunk = 16;
    parallelRows(0, (int)((npix + chunk - 1) / chunk), threads, [&](int chunk_id) {
        uint64_t local = 0;
        const int64_t p_end = std::min<int64_t>(npix, (int64_t)(chunk_id + 1) * chunk);
        for (int64_t q = (int64_t)chunk_id * chunk; q < p_end; ++q) {
            const int j = r0 + (int)(q / s.width), i = (int)(q % s.width);
            PixelOut o = ref ? renderPixelReference(s, i, j, prm->spp, prm->seed) : renderPixelConfig(s, i, j, *prm);
            size_t off = (size_t)j * s.width + i;
            rgb[3 * off] = o.rgb.x;
            rgb[3 * off + 1] = o.rgb.y;
            rgb[3 * off + 2] = o.rgb.z;
            if (rgba8) {
                double c[3] = {std::sqrt(o.rgb.x), std::sqrt(o.rgb.y), std::sqrt(o.rgb.z)};
                for (int k = 0; k < 3; ++k) {
                    double x = c[k] > 1.0 ? 1.0 : (c[k] < 0.0 ? 0.0 : c[k]);
                    rgba8[4 * off + k] = (uint8_t)(254.99 * x);
                }
                rgba8[4 * off + 3] = 255;
            }
            if (gbuf) {
                double g[8] = {o.gN.x, o.gN.y, o.gN.z, o.gDepth, o.gAlbedo.x, o.gAlbedo.y, o.gAlbedo.z, o.gVar};
                std::memcpy(gbuf + 8 * off, g, sizeof g);
            }
            local += o.rays;
        }
        total += local;
    });
    return total.load();
}

// getObject (Render.cu:485-496): the primitive hit by the ray through the centre of pixel (x, y)
// (Camera::getSampleRay, Camera.cuh:44-48) with traverseIterative's default interval, or -1.
ORC_API int orc_pick(void* p, int x, int y)
{
    Handle* h = (Handle*)p;
    const Scene& s = h->ref;
    V3 px = s.pixelCenter + (double)x * s.dh + (double)y * s.dv;
    Ray ray = {s.lookFrom, px - s.lookFrom};
    HitRecord rec;
    int id = traverse(s, ray, rec);
    return (id >= 0 && rec.material != nullptr) ? id : -1;
}

// changeMaterial (Render.cu:498-522) over primitives [first, end) of both estimators' copies:
// spheres and triangles take (alphaX, alphaY) and Opaque, or SpecularDielectric when glass;
// lights are skipped.
ORC_API void orc_set_material(void* p, int first, int end, double alphaX, double alphaY, int glass)
{
    Handle* h = (Handle*)p;
    Scene* both[2] = {&h->ref, &h->cfg};
    for (Scene* s : both) {
        const int n = (int)s->prims.size();
        for (int i = first < 0 ? 0 : first; i < end && i < n; ++i) {
            Prim& q = s->prims[i];
            if (q.kind == K_LIGHT) continue;
            q.mat.ax = alphaX;
            q.mat.ay = alphaY;
            q.mat.type = glass ? M_SPEC : M_OPAQUE;
        }
    }
}

// Renders like orc_render (rgb only) while counting, for every closest-hit query the render
// makes, the internal-node visits and primitive tests of the ordered, pruned traversal of the
// binary LBVH.  out[0] = queries, out[1] = internal visits, out[2] = primitive tests.
ORC_API void orc_render_visit_counts(void* p, const cpt_render_params* prm, int threads, uint64_t* out)
{
    Handle* h = (Handle*)p;
    bool ref = prm->estimator == CPT_ESTIMATOR_REFERENCE;
    const Scene& s = ref ? h->ref : h->cfg;
    int r0 = prm->row_begin, r1 = prm->row_end;
    if (r0 == 0 && r1 == 0) r1 = s.height;
    std::atomic<uint64_t> q(0), vi(0), vl(0);
    parallelRows(r0, r1, threads, [&](int j) {
        VisitCounts c = {0, 0, 0};
        g_visit = &c;
        for (int i = 0; i < s.width; ++i) {
            if (ref)
                renderPixelReference(s, i, j, prm->spp, prm->seed);
            else
                renderPixelConfig(s, i, j, *prm);
        }
        g_visit = nullptr;
        q += c.rays;
        vi += c.vInt;
        vl += c.vLeaf;
    });
    out[0] = q.load();
    out[1] = vi.load();
    out[2] = vl.load();
}
