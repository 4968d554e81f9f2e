// ini.cpp — scene files: the reference's INI format (IniParser.cpp:3-128) and the scene
// assembly of Scene::init (Scene.cuh:72-145), producing a cpt_scene_desc on the host.
//
// Parsing follows the reference line by line: a line that is empty or starts with ';' is
// skipped; "[Name]" opens a section (Light/Sphere/Floor/Mesh append a default object);
// "key=value" splits at the first '=', with no trimming; unknown keys are ignored; colours
// are integers divided by 255; vectors are "(x, y, z)".  Where the reference would throw
// from std::stoi/std::stod (and terminate), this returns CPT_ERR_PARSE.
//
// Backward-compatible extensions (ignored by the reference): type=Lambertian and the keys
// eta=, sigmaT=, albedo= in [Sphere], [Floor] and [Mesh]; usingNV= in [Mesh].
//
// [Mesh] loads a Wavefront OBJ like Mesh::loadFromFile (ObjLoader.cuh:39-163): vertices are
// read as float (tinyobjloader's real_t), rotated about y by `rotation` degrees, scaled, fed
// to the scene bounds, then translated by `center`.  Polygons are fanned into triangles
// (the reference's loader triangulates; concave polygons may split differently).  Each corner
// takes its vt texture coordinate ((0, 0) without one, ObjLoader.cuh:119-134).  Vertex normals
// (vn) are used only with the extension key usingNV=1: the loader reads them when its usingNV
// flag is set (ObjLoader.cuh:136-151), which Scene::init never sets (Scene.cuh:89), so by default
// meshes are flat-shaded as in the reference.
//
// Images (texture= in [Mesh], skyBox= in [Camera]) are read where the reference calls stbi_load
// (Scene.cuh:244-253, Camera.cu:33-39).  This build has no stb_image; it reads binary PPM (P6,
// 8-bit) files, the format the library's own image writer produces.  A file that cannot be read
// leaves the mesh untextured / the sky at the background colour, as a failed stbi_load does in
// the reference (the path is recorded as a warning).
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "cpt_internal.h"

namespace cpt {

namespace {

const double INF_D = 999999.0;
const double PI_D = 3.14159265358979323846;

struct V3d { double x, y, z; };

struct LightInfo { V3d center{0, 0, 0}; double width = 0, height = 0; V3d normal{0, 0, 1}; V3d color{1, 1, 1}; bool visible = true; };
struct MatInfo { V3d color{1, 1, 1}; double alphaX = 0.5, alphaY = 0.5; int type = CPT_M_OPAQUE; double eta = 1.51, sigmaT = 0.0, albedo = 0.0; };
struct SphereInfo { V3d center{0, 0, 0}; double radius = 0; MatInfo m; };
struct FloorInfo { V3d lt{0, 0, 0}, rt{0, 0, 0}, lb{0, 0, 0}, rb{0, 0, 0}; MatInfo m; };
struct MeshInfo { std::string path, texture; V3d center{0, 0, 0}; MatInfo m; double rotation = 0, scale = 1; bool usingNV = false; };
struct CameraInfo {   // IniParser.h:14-24
    V3d background{0, 0, 0};
    double width = 0, aspectRatio = 16.0 / 9.0;
    V3d lookFrom{0, 0, 1}, lookAt{0, 0, 0};
    double vFov = 90.0;
    std::string skyBox;
};

struct ParseError { std::string msg; };

V3d parse_vec3(const std::string& s)   // IniParser.cpp:98-105
{
    V3d v{0, 0, 0};
    std::istringstream ss(s);
    char discard;
    ss >> discard >> v.x >> discard >> v.y >> discard >> v.z >> discard;
    return v;
}

V3d parse_color(const std::string& s)   // IniParser.cpp:107-118
{
    std::istringstream ss(s);
    int x = 0, y = 0, z = 0;
    char discard;
    ss >> discard >> x >> discard >> y >> discard >> z >> discard;
    return V3d{x / 255.0, y / 255.0, z / 255.0};
}

int parse_material(const std::string& s)   // IniParser.cpp:120-128
{
    if (s == "Light") return CPT_M_LIGHT;
    if (s == "Opaque") return CPT_M_OPAQUE;
    if (s == "SpecularDielectric") return CPT_M_SPECULAR_DIELECTRIC;
    if (s == "RoughDielectric") return CPT_M_ROUGH_DIELECTRIC;
    if (s == "Volume") return CPT_M_VOLUME;
    if (s == "Lambertian") return CPT_M_LAMBERTIAN;
    return CPT_M_OPAQUE;
}

double to_d(const std::string& key, const std::string& v)
{
    try {
        return std::stod(v);
    } catch (...) {
        throw ParseError{"bad number for '" + key + "': '" + v + "'"};
    }
}

int to_i(const std::string& key, const std::string& v)
{
    try {
        return std::stoi(v);
    } catch (...) {
        throw ParseError{"bad integer for '" + key + "': '" + v + "'"};
    }
}

bool material_key(MatInfo& m, const std::string& key, const std::string& value)
{
    if (key == "color") m.color = parse_color(value);
    else if (key == "alphaX") m.alphaX = to_d(key, value);
    else if (key == "alphaY") m.alphaY = to_d(key, value);
    else if (key == "type") m.type = parse_material(value);
    else if (key == "eta") m.eta = to_d(key, value);
    else if (key == "sigmaT") m.sigmaT = to_d(key, value);
    else if (key == "albedo") m.albedo = to_d(key, value);
    else return false;
    return true;
}

}  // namespace

struct IniScene {
    CameraInfo camera;
    std::vector<LightInfo> lights_in;
    std::vector<SphereInfo> spheres_in;
    std::vector<FloorInfo> floors_in;
    std::vector<MeshInfo> meshes_in;
    bool has_cloth = false;
    // assembled description
    std::vector<cpt_light> lights;
    std::vector<cpt_sphere> spheres;
    std::vector<cpt_material> mats;
    std::vector<double> tri;      // 9 per triangle
    std::vector<uint32_t> tri_mat;
    std::vector<float> tri_uv;    // 6 per triangle
    std::vector<float> tri_n;     // 9 per triangle
    bool any_uv = false, any_normal = false;
    std::vector<std::vector<uint8_t>> images;   // texture texels (RGB8), then the sky's
    std::vector<cpt_image> textures;
    std::vector<uint8_t> sky_rgb;
    cpt_image sky{0, 0, nullptr};
    double bmin[3], bmax[3];
    std::vector<std::string> warnings;   // mesh files that could not be opened
    cpt_scene_desc desc;
};

namespace {

uint32_t add_material(IniScene& s, const MatInfo& m)
{
    cpt_material c;
    std::memset(&c, 0, sizeof c);
    c.color[0] = m.color.x; c.color[1] = m.color.y; c.color[2] = m.color.z;
    c.alpha_x = m.alphaX; c.alpha_y = m.alphaY;
    c.type = m.type;
    c.eta = m.eta; c.sigma_t = m.sigmaT; c.albedo = m.albedo;
    s.mats.push_back(c);
    return (uint32_t)(s.mats.size() - 1);
}

struct Corner {
    float uv[2];
    float n[3];
};

void push_tri(IniScene& s, V3d a, V3d b, V3d c, uint32_t mi, const Corner* k = nullptr)
{
    double v[9] = {a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z};
    s.tri.insert(s.tri.end(), v, v + 9);
    s.tri_mat.push_back(mi);
    for (int i = 0; i < 3; ++i) {
        s.tri_uv.push_back(k ? k[i].uv[0] : 0.f);
        s.tri_uv.push_back(k ? k[i].uv[1] : 0.f);
        for (int a2 = 0; a2 < 3; ++a2) s.tri_n.push_back(k ? k[i].n[a2] : 0.f);
    }
}

// One face corner of an OBJ f record: vertex, texture-coordinate and normal indices (-1: none).
struct ObjIndex {
    long v, vt, vn;
};

struct ObjData {
    std::vector<float> v, vt, vn;   // 3, 2, 3 floats per record
    std::vector<std::vector<ObjIndex>> faces;
};

// OBJ index: 1-based, or negative = relative to the records read so far; -1 when absent.
bool obj_index(const std::string& tok, long count, long& out)
{
    if (tok.empty()) {
        out = -1;
        return true;
    }
    long i = std::strtol(tok.c_str(), nullptr, 10);
    i = i < 0 ? count + i : i - 1;
    out = i;
    return i >= 0 && i < count;
}

// Minimal Wavefront OBJ reader: v, vt, vn and f records (v, v/vt, v//vn, v/vt/vn; negative
// indices); other records are ignored.
cpt_status load_obj(const std::string& path, ObjData& o)
{
    std::ifstream f(path);
    if (!f) return fail(CPT_ERR_IO, "cannot open mesh file " + path);
    std::string line;
    while (std::getline(f, line)) {
        if (line.size() < 2) continue;
        std::istringstream ss(line);
        std::string tag;
        ss >> tag;
        if (tag == "v" || tag == "vn") {
            double x = 0, y = 0, z = 0;
            ss >> x >> y >> z;
            std::vector<float>& dst = tag == "v" ? o.v : o.vn;
            dst.push_back((float)x);
            dst.push_back((float)y);
            dst.push_back((float)z);
        } else if (tag == "vt") {
            double u = 0, v = 0;
            ss >> u >> v;
            o.vt.push_back((float)u);
            o.vt.push_back((float)v);
        } else if (tag == "f") {
            std::string tok;
            std::vector<ObjIndex> face;
            while (ss >> tok) {
                std::string part[3];
                size_t a = tok.find('/');
                part[0] = tok.substr(0, a);
                if (a != std::string::npos) {
                    size_t b = tok.find('/', a + 1);
                    part[1] = tok.substr(a + 1, b == std::string::npos ? std::string::npos : b - a - 1);
                    if (b != std::string::npos) part[2] = tok.substr(b + 1);
                }
                ObjIndex ix;
                if (part[0].empty() || !obj_index(part[0], (long)(o.v.size() / 3), ix.v) ||
                    !obj_index(part[1], (long)(o.vt.size() / 2), ix.vt) ||
                    !obj_index(part[2], (long)(o.vn.size() / 3), ix.vn))
                    return fail(CPT_ERR_PARSE, "bad face index in " + path);
                face.push_back(ix);
            }
            if (face.size() >= 3) o.faces.push_back(face);
        }
    }
    return CPT_OK;
}

// Binary PPM (P6, maxval 255) into RGB8 texels, rows in file order.
bool load_ppm(const std::string& path, std::vector<uint8_t>& rgb, int& w, int& h)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    auto token = [&](std::string& t) {
        t.clear();
        int c;
        while ((c = f.get()) != EOF) {
            if (c == '#') {
                while ((c = f.get()) != EOF && c != '\n') {}
                continue;
            }
            if (std::isspace(c)) {
                if (!t.empty()) return true;
                continue;
            }
            t.push_back((char)c);
        }
        return !t.empty();
    };
    std::string magic, sw, sh, smax;
    if (!token(magic) || magic != "P6" || !token(sw) || !token(sh) || !token(smax)) return false;
    w = std::atoi(sw.c_str());
    h = std::atoi(sh.c_str());
    if (w <= 0 || h <= 0 || std::atoi(smax.c_str()) != 255 || (long long)w * h > (1ll << 28)) return false;
    rgb.resize(3 * (size_t)w * h);
    f.read((char*)rgb.data(), (std::streamsize)rgb.size());
    return (size_t)f.gcount() == rgb.size();
}

cpt_status add_mesh(IniScene& s, const MeshInfo& m)   // Scene::addMeshes (Scene.cuh:232-270)
{
    ObjData obj;
    uint32_t mi = add_material(s, m.m);
    if (!m.texture.empty()) {   // stbi_load (Scene.cuh:244-253); unreadable: untextured
        std::vector<uint8_t> rgb;
        int w = 0, h = 0;
        if (load_ppm(m.texture, rgb, w, h)) {
            s.images.push_back(std::move(rgb));
            s.textures.push_back(cpt_image{w, h, nullptr});
            s.mats[mi].texture = (int32_t)s.textures.size();
        } else {
            s.warnings.push_back(m.texture);
        }
    }
    cpt_status st = load_obj(m.path, obj);
    if (st == CPT_ERR_IO) {
        // Mesh::loadMesh prints the loader error and leaves the mesh empty (ObjLoader.cuh:66-70);
        // the scene still loads.  The message stays readable through cpt_last_error_string.
        s.warnings.push_back(m.path);
        return CPT_OK;
    }
    if (st != CPT_OK) return st;
    double theta = m.rotation * PI_D / 180.0;   // ObjLoader.cuh:72-77
    double c = std::cos(theta), sn = std::sin(theta);
    const std::vector<float>& v = obj.v;
    auto xform = [&](long i) {
        double x = v[3 * i], y = v[3 * i + 1], z = v[3 * i + 2];
        // Dot(p, (c,0,s)), Dot(p, (0,1,0)), Dot(p, (-s,0,c)), then * scale (ObjLoader.cuh:101-106)
        double rx = x * c + y * 0.0 + z * sn;
        double ry = x * 0.0 + y * 1.0 + z * 0.0;
        double rz = x * -sn + y * 0.0 + z * c;
        V3d p{rx * m.scale, ry * m.scale, rz * m.scale};
        s.bmin[0] = std::min(s.bmin[0], p.x); s.bmin[1] = std::min(s.bmin[1], p.y); s.bmin[2] = std::min(s.bmin[2], p.z);
        s.bmax[0] = std::max(s.bmax[0], p.x); s.bmax[1] = std::max(s.bmax[1], p.y); s.bmax[2] = std::max(s.bmax[2], p.z);
        return V3d{p.x + m.center.x, p.y + m.center.y, p.z + m.center.z};   // Mesh::transform
    };
    auto corner = [&](const ObjIndex& ix) {
        Corner c{{0.f, 0.f}, {0.f, 0.f, 0.f}};
        if (ix.vt >= 0) {
            c.uv[0] = obj.vt[2 * ix.vt];
            c.uv[1] = obj.vt[2 * ix.vt + 1];
            s.any_uv = true;
        }
        if (m.usingNV && ix.vn >= 0) {
            for (int a = 0; a < 3; ++a) c.n[a] = obj.vn[3 * ix.vn + a];
            s.any_normal = true;
        }
        return c;
    };
    for (const auto& f : obj.faces)
        for (size_t k = 1; k + 1 < f.size(); ++k) {
            V3d a = xform(f[0].v), b = xform(f[k].v), cc = xform(f[k + 1].v);
            Corner cs[3] = {corner(f[0]), corner(f[k]), corner(f[k + 1])};
            push_tri(s, a, b, cc, mi, cs);
        }
    return CPT_OK;
}

cpt_status parse_file(const char* path, IniScene& s)   // IniParser::Parse (IniParser.cpp:3-96)
{
    std::ifstream file(path);
    if (!file) return fail(CPT_ERR_IO, std::string("unable to open file ") + path);
    std::string line, section;
    try {
        while (std::getline(file, line)) {
            if (line.empty() || line[0] == ';') continue;
            if (line[0] == '[') {
                section = line.substr(1, line.find(']') - 1);
                if (section == "Light") s.lights_in.push_back(LightInfo());
                else if (section == "Sphere") s.spheres_in.push_back(SphereInfo());
                else if (section == "Floor") s.floors_in.push_back(FloorInfo());
                else if (section == "Mesh") s.meshes_in.push_back(MeshInfo());
                continue;
            }
            size_t eq = line.find('=');
            if (eq == std::string::npos) continue;
            std::string key = line.substr(0, eq), value = line.substr(eq + 1);
            if (section == "Camera") {
                CameraInfo& c = s.camera;
                if (key == "background") c.background = parse_color(value);
                else if (key == "skyBox") c.skyBox = value;
                else if (key == "width") c.width = to_i(key, value);
                else if (key == "aspectRatio") c.aspectRatio = to_d(key, value);
                else if (key == "lookFrom") c.lookFrom = parse_vec3(value);
                else if (key == "lookAt") c.lookAt = parse_vec3(value);
                else if (key == "vFov") c.vFov = to_d(key, value);
            } else if (section == "Light") {
                LightInfo& L = s.lights_in.back();
                if (key == "center") L.center = parse_vec3(value);
                else if (key == "width") L.width = to_d(key, value);
                else if (key == "height") L.height = to_d(key, value);
                else if (key == "normal") L.normal = parse_vec3(value);
                else if (key == "color") L.color = parse_color(value);
                else if (key == "visible") L.visible = to_i(key, value) != 0;
            } else if (section == "Sphere") {
                SphereInfo& S = s.spheres_in.back();
                if (key == "center") S.center = parse_vec3(value);
                else if (key == "radius") S.radius = to_d(key, value);
                else material_key(S.m, key, value);
            } else if (section == "Floor") {
                FloorInfo& F = s.floors_in.back();
                if (key == "lt") F.lt = parse_vec3(value);
                else if (key == "rt") F.rt = parse_vec3(value);
                else if (key == "lb") F.lb = parse_vec3(value);
                else if (key == "rb") F.rb = parse_vec3(value);
                else material_key(F.m, key, value);
            } else if (section == "Mesh") {
                MeshInfo& M = s.meshes_in.back();
                if (key == "path") M.path = value;
                else if (key == "texture") M.texture = value;
                else if (key == "center") M.center = parse_vec3(value);
                else if (key == "rotation") M.rotation = to_d(key, value);
                else if (key == "scale") M.scale = to_d(key, value);
                else if (key == "usingNV") M.usingNV = to_i(key, value) != 0;
                else material_key(M.m, key, value);
            } else if (section == "Cloth") {
                s.has_cloth = true;
            }
        }
    } catch (const ParseError& e) {
        return fail(CPT_ERR_PARSE, std::string(path) + ": " + e.msg);
    }
    return CPT_OK;
}

}  // namespace

cpt_status ini_load(const char* path, IniScene** out)
{
    if (!path || !out) return fail(CPT_ERR_INVALID_ARGUMENT, "cpt_ini_load: null argument");
    IniScene* s = new IniScene();
    cpt_status st = parse_file(path, *s);
    if (st != CPT_OK) { delete s; return st; }
    for (int a = 0; a < 3; ++a) { s->bmin[a] = INF_D; s->bmax[a] = -INF_D; }   // Scene.cuh:61-62
    for (const auto& L : s->lights_in) {   // addOneLight
        cpt_light l;
        std::memset(&l, 0, sizeof l);
        l.center[0] = L.center.x; l.center[1] = L.center.y; l.center[2] = L.center.z;
        l.normal[0] = L.normal.x; l.normal[1] = L.normal.y; l.normal[2] = L.normal.z;
        l.width = L.width; l.height = L.height;
        l.color[0] = L.color.x; l.color[1] = L.color.y; l.color[2] = L.color.z;
        l.visible = L.visible ? 1 : 0;
        s->lights.push_back(l);
    }
    for (const auto& S : s->spheres_in) {   // addOneSphere
        cpt_sphere sp;
        std::memset(&sp, 0, sizeof sp);
        sp.center[0] = S.center.x; sp.center[1] = S.center.y; sp.center[2] = S.center.z;
        sp.radius = S.radius;
        sp.material = add_material(*s, S.m);
        s->spheres.push_back(sp);
    }
    for (const auto& F : s->floors_in) {   // addFloor: (lt, lb, rt), (rt, lb, rb) (Device.cuh:42-43)
        uint32_t mi = add_material(*s, F.m);
        push_tri(*s, F.lt, F.lb, F.rt, mi);
        push_tri(*s, F.rt, F.lb, F.rb, mi);
    }
    for (const auto& M : s->meshes_in) {
        st = add_mesh(*s, M);
        if (st != CPT_OK) { delete s; return st; }
    }
    if (s->mats.empty()) add_material(*s, MatInfo());
    if (!s->camera.skyBox.empty()) {   // Camera.cu:33-39; unreadable: the background colour
        int w = 0, h = 0;
        if (load_ppm(s->camera.skyBox, s->sky_rgb, w, h))
            s->sky = cpt_image{w, h, s->sky_rgb.data()};
        else
            s->warnings.push_back(s->camera.skyBox);
    }
    for (size_t i = 0; i < s->textures.size(); ++i) s->textures[i].rgb = s->images[i].data();
    cpt_scene_desc& d = s->desc;
    std::memset(&d, 0, sizeof d);
    d.num_lights = (uint32_t)s->lights.size();
    d.lights = s->lights.data();
    d.num_spheres = (uint32_t)s->spheres.size();
    d.spheres = s->spheres.data();
    d.num_triangles = (uint32_t)s->tri_mat.size();
    d.tri_vertices_f64 = s->tri.empty() ? nullptr : s->tri.data();
    d.tri_material = s->tri_mat.empty() ? nullptr : s->tri_mat.data();
    d.num_materials = (uint32_t)s->mats.size();
    d.materials = s->mats.data();
    d.tri_uvs = s->any_uv && !s->tri_uv.empty() ? s->tri_uv.data() : nullptr;
    d.tri_normals = s->any_normal && !s->tri_n.empty() ? s->tri_n.data() : nullptr;
    d.num_textures = (uint32_t)s->textures.size();
    d.textures = s->textures.empty() ? nullptr : s->textures.data();
    d.sky = s->sky;
    for (int a = 0; a < 3; ++a) { d.bounds_min[a] = s->bmin[a]; d.bounds_max[a] = s->bmax[a]; }
    const CameraInfo& c = s->camera;   // main.cu:26-37
    d.camera.width = (int)c.width;
    d.camera.aspect_ratio = c.aspectRatio;
    double h = d.camera.width / c.aspectRatio;
    d.camera.height = h < 1 ? 1 : (int)h;
    d.camera.look_from[0] = c.lookFrom.x; d.camera.look_from[1] = c.lookFrom.y; d.camera.look_from[2] = c.lookFrom.z;
    d.camera.look_at[0] = c.lookAt.x; d.camera.look_at[1] = c.lookAt.y; d.camera.look_at[2] = c.lookAt.z;
    d.camera.vfov_deg = c.vFov;
    d.camera.background[0] = c.background.x; d.camera.background[1] = c.background.y;
    d.camera.background[2] = c.background.z;
    *out = s;
    return CPT_OK;
}

const cpt_scene_desc* ini_desc(const IniScene* s) { return &s->desc; }
bool ini_has_cloth(const IniScene* s) { return s->has_cloth; }
void ini_free(IniScene* s) { delete s; }

}  // namespace cpt
