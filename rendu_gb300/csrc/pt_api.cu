// C-ABI of the path tracer (include/rendu_gb300.h, pt_*): scene intake, upload
// (PathTracer::PathTracer, PathTracer.cpp:11-21 of kosua20/Rendu) and the render driver
// (PathTracer::render, PathTracer.cpp:159-299).
#include <cmath>
#include <cstring>
#include <string>

#include "pt_scene.hpp"

using namespace rgb;

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

int arg_error(const char *msg) {
    set_error(msg);
    return RT_ERR_ARG;
}

// Validation shared by pt_render and the batch jobs (PathTracer.cpp:162-173).
int check_job(const pt_scene *s, uint32_t samples, uint32_t width, uint32_t height, uint32_t components) {
    if (!s->committed) {
        set_error("pt_scene_commit must be called after the last scene change");
        return RT_ERR_STATE;
    }
    if (width == 0 || height == 0) return arg_error("empty image");
    if (components < 3) return arg_error("the image needs at least 3 components (PathTracer.cpp:166-168)");
    if (samples == 0) return arg_error("samples must be at least 1");
    if ((uint64_t)width * height >= (1ull << 28)) return arg_error("image too large");
    return RT_OK;
}

template <class T>
int upload(DevBuf &b, const std::vector<T> &v, cudaStream_t st) {
    if (b.reserve(sizeof(T) * (v.empty() ? 1 : v.size())) != RT_OK) return RT_ERR_OOM;
    if (!v.empty()) RT_CUDA_TRY(cudaMemcpyAsync(b.ptr, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st));
    return RT_OK;
}

struct V3 {
    float x, y, z;
};
V3 vnormalize(V3 v) {
    const float s = 1.0f / std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    return {v.x * s, v.y * s, v.z * s};
}

// inverse(transpose(mat3(model))) as a row-major 3x3 acting on column vectors.
void normal_matrix(const float *m, float out[9]) {
    double a[3][3];  // a[r][c] = model column c, row r
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) a[r][c] = m[4 * c + r];
    const double det = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
                       a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
    double inv[3][3];
    inv[0][0] = (a[1][1] * a[2][2] - a[1][2] * a[2][1]) / det;
    inv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
    inv[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / det;
    inv[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) / det;
    inv[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / det;
    inv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
    inv[2][0] = (a[1][0] * a[2][1] - a[1][1] * a[2][0]) / det;
    inv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
    inv[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / det;
    // (M^-1)^T
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) out[3 * r + c] = (float)inv[c][r];
}

}  // namespace

extern "C" {

int pt_scene_create(pt_scene **out, int device) {
    clear_error();
    if (!out) return arg_error("null output pointer");
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        set_error("CUDA device " + std::to_string(device) + " is not available");
        return RT_ERR_CUDA;
    }
    pt_scene *s = new pt_scene();
    s->device = device;
    *out = s;
    return RT_OK;
}

int pt_scene_destroy(pt_scene *s) {
    if (!s) return RT_OK;
    DeviceGuard g(s->device);
    if (s->rc) rt_destroy(s->rc);
    for (DevBuf *b : {&s->d_positions, &s->d_emitters, &s->d_emitter_cdf, &s->d_env_marg, &s->d_env_cond,
                      &s->d_env_func, &s->d_objects, &s->d_meshes, &s->d_materials, &s->d_tex, &s->d_texels, &s->d_normals,
                      &s->d_tangents, &s->d_bitangents, &s->d_uvs, &s->d_indices, &s->d_lights, &s->d_sky})
        b->release();
    s->engine.reset();
    delete s;
    return RT_OK;
}

int pt_scene_add_texture(pt_scene *s, uint32_t width, uint32_t height, uint32_t channels, const float *pixels,
                         uint32_t *tex_id) {
    clear_error();
    if (!s || !pixels) return arg_error("null argument");
    if (width == 0 || height == 0 || channels < 1 || channels > 4) return arg_error("bad texture size or channels");
    HostTex t;
    t.w = width;
    t.h = height;
    t.rgba.resize((size_t)width * height * 4);
    for (size_t p = 0; p < (size_t)width * height; ++p)
        for (uint32_t c = 0; c < 4; ++c) t.rgba[4 * p + c] = c < channels ? pixels[channels * p + c] : (c == 3 ? 1.0f : 0.0f);
    s->textures.push_back(std::move(t));
    if (tex_id) *tex_id = (uint32_t)(s->textures.size() - 1);
    s->committed = false;
    return RT_OK;
}

int pt_scene_add_mesh(pt_scene *s, const pt_mesh_desc *m, uint32_t *mesh_id) {
    clear_error();
    if (!s || !m) return arg_error("null argument");
    if (!m->positions || !m->normals || !m->tangents || !m->bitangents || (m->index_count && !m->indices))
        return arg_error("the path tracer requires positions, normals, tangents and bitangents (PathTracer.cpp:14-16)");
    if (m->index_count % 3) return arg_error("index_count must be a multiple of 3");
    for (size_t i = 0; i < m->index_count; ++i)
        if (m->indices[i] >= m->vertex_count) return arg_error("mesh index out of range");
    HostMesh h;
    const size_t nv = m->vertex_count;
    h.pos.assign(m->positions, m->positions + 3 * nv);
    h.nrm.assign(m->normals, m->normals + 3 * nv);
    h.tan.assign(m->tangents, m->tangents + 3 * nv);
    h.bit.assign(m->bitangents, m->bitangents + 3 * nv);
    if (m->texcoords) h.uv.assign(m->texcoords, m->texcoords + 2 * nv);
    h.idx.assign(m->indices, m->indices + m->index_count);
    s->meshes.push_back(std::move(h));
    if (mesh_id) *mesh_id = (uint32_t)(s->meshes.size() - 1);
    s->committed = false;
    return RT_OK;
}

int pt_scene_add_material(pt_scene *s, const pt_material_desc *d, uint32_t *material_id) {
    clear_error();
    if (!s || !d) return arg_error("null argument");
    if (d->type < 0 || d->type > 10) return arg_error("unknown material type");
    for (int k = 0; k < 3; ++k)
        if (d->tex[k] >= s->textures.size()) return arg_error("material texture id out of range");
    s->materials.push_back(*d);
    if (material_id) *material_id = (uint32_t)(s->materials.size() - 1);
    s->committed = false;
    return RT_OK;
}

int pt_scene_add_object(pt_scene *s, uint32_t mesh_id, uint32_t material_id, const float *model, uint32_t *object_id) {
    clear_error();
    if (!s) return arg_error("null scene");
    if (mesh_id >= s->meshes.size() || material_id >= s->materials.size()) return arg_error("mesh or material id out of range");
    HostObject o;
    o.mesh = mesh_id;
    o.material = material_id;
    for (int k = 0; k < 16; ++k) o.model[k] = model ? model[k] : ((k % 5) == 0 ? 1.0f : 0.0f);
    s->objects.push_back(o);
    if (object_id) *object_id = (uint32_t)(s->objects.size() - 1);
    s->committed = false;
    return RT_OK;
}

int pt_scene_add_light(pt_scene *s, const pt_light_desc *l) {
    clear_error();
    if (!s || !l) return arg_error("null argument");
    if (l->type < PT_LIGHT_POINT || l->type > PT_LIGHT_SPOT) return arg_error("unknown light type");
    s->lights.push_back(*l);
    s->committed = false;
    return RT_OK;
}

int pt_scene_set_background(pt_scene *s, int32_t mode, const float *color, const uint32_t *tex) {
    clear_error();
    if (!s) return arg_error("null scene");
    if (mode == PT_BG_COLOR) {
        if (!color) return arg_error("COLOR background needs a colour");
        std::memcpy(s->bg_color, color, sizeof(s->bg_color));
    } else if (mode == PT_BG_IMAGE || mode == PT_BG_SKYBOX) {
        const int n = mode == PT_BG_IMAGE ? 1 : 6;
        if (!tex) return arg_error("background needs texture ids");
        for (int k = 0; k < n; ++k) {
            if (tex[k] >= s->textures.size()) return arg_error("background texture id out of range");
            s->bg_tex[k] = tex[k];
        }
    } else if (mode == PT_BG_ATMOSPHERE) {
        // Sky::decode / Sky::update normalise the sun direction (Sky.cpp:16, 35).
        if (!color) return arg_error("ATMOSPHERE background needs the sun direction");
        const float d = (color[0] * color[0] + color[1] * color[1]) + color[2] * color[2];
        if (!(d > 0.0f) || !std::isfinite(d)) return arg_error("invalid sun direction");
        const float k = 1.0f / std::sqrt(d);
        for (int c = 0; c < 3; ++c) s->sun[c] = color[c] * k;
    } else {
        return arg_error("unsupported background mode");
    }
    s->bg_mode = mode;
    s->committed = false;
    return RT_OK;
}

int pt_scene_set_sky_table(pt_scene *s, const float *rgba, uint32_t width, uint32_t height) {
    clear_error();
    if (!s) return arg_error("null scene");
    if (!rgba) {
        s->sky_table.clear();
        s->sky_w = s->sky_h = 0;
    } else {
        if (width == 0 || height == 0 || (uint64_t)width * height > (1u << 24)) return arg_error("invalid table size");
        s->sky_table.assign(rgba, rgba + 4 * (size_t)width * height);
        s->sky_w = width;
        s->sky_h = height;
    }
    s->committed = false;
    return RT_OK;
}

int pt_scene_set_environment(pt_scene *s, uint32_t tex_id, float intensity) {
    clear_error();
    if (!s) return arg_error("null scene");
    if (tex_id >= s->textures.size()) return arg_error("environment texture id out of range");
    if (!(intensity >= 0.0f)) return arg_error("environment intensity must be >= 0");
    s->env_tex = (int)tex_id;
    s->env_intensity = intensity;
    s->committed = false;
    return RT_OK;
}

int pt_scene_commit(pt_scene *s) {
    clear_error();
    if (!s) return arg_error("null scene");
    DeviceGuard g(s->device);
    if (s->rc) rt_destroy(s->rc);
    s->rc = nullptr;
    int r = rt_create(&s->rc, s->device);
    if (r != RT_OK) return r;
    // Every object's mesh is added in object order: meshId == object index (PathTracer.cpp:16-18).
    for (const HostObject &o : s->objects) {
        const HostMesh &m = s->meshes[o.mesh];
        r = rt_add_mesh(s->rc, m.pos.data(), m.pos.size() / 3, m.idx.data(), m.idx.size(), o.model, nullptr);
        if (r != RT_OK) return r;
    }
    r = rt_update_hierarchy(s->rc);
    if (r != RT_OK) return r;
    cudaStream_t st = s->rc->stream;

    std::vector<PtMesh> meshes(s->meshes.size());
    std::vector<float> posp, nrm, tan, bit, uv;
    std::vector<uint32_t> idx;
    for (size_t k = 0; k < s->meshes.size(); ++k) {
        const HostMesh &m = s->meshes[k];
        meshes[k].first_vertex = (uint32_t)(nrm.size() / 3);
        meshes[k].first_index = (uint32_t)idx.size();
        meshes[k].has_uv = m.uv.empty() ? 0 : 1;
        posp.insert(posp.end(), m.pos.begin(), m.pos.end());
        nrm.insert(nrm.end(), m.nrm.begin(), m.nrm.end());
        tan.insert(tan.end(), m.tan.begin(), m.tan.end());
        bit.insert(bit.end(), m.bit.begin(), m.bit.end());
        if (m.uv.empty()) uv.resize(uv.size() + 2 * (m.pos.size() / 3), 0.0f);
        else uv.insert(uv.end(), m.uv.begin(), m.uv.end());
        idx.insert(idx.end(), m.idx.begin(), m.idx.end());
    }
    std::vector<PtObject> objects(s->objects.size());
    bool any_masked = false;
    for (size_t k = 0; k < s->objects.size(); ++k) {
        const HostObject &o = s->objects[k];
        objects[k].mesh = o.mesh;
        objects[k].material = o.material;
        objects[k].first_tri = (uint32_t)s->rc->meshes[k].first_tri;
        // Object::Object: texture coordinates are used when the mesh had some (Object.cpp:4-8).
        objects[k].use_uv = meshes[o.mesh].has_uv;
        normal_matrix(o.model, objects[k].invtp);
        if (s->materials[o.material].masked) any_masked = true;
    }
    std::vector<PtMaterial> mats(s->materials.size());
    for (size_t k = 0; k < mats.size(); ++k) {
        mats[k].type = s->materials[k].type;
        mats[k].masked = s->materials[k].masked ? 1 : 0;
        for (int t = 0; t < 3; ++t) mats[k].tex[t] = s->materials[k].tex[t];
    }
    std::vector<PtTex> texd(s->textures.size());
    std::vector<float> texels;
    for (size_t k = 0; k < texd.size(); ++k) {
        const HostTex &t = s->textures[k];
        texd[k].w = t.w;
        texd[k].h = t.h;
        texd[k].offset = texels.size() / 4;
        bool constant = true;
        for (size_t p = 4; p < t.rgba.size() && constant; ++p) constant = t.rgba[p] == t.rgba[p % 4];
        texd[k].constant = constant ? 1 : 0;
        texd[k].value = make_float4(t.rgba[0], t.rgba[1], t.rgba[2], t.rgba[3]);
        texels.insert(texels.end(), t.rgba.begin(), t.rgba.end());
    }
    std::vector<PtLight> lights(s->lights.size());
    bool any_shadow = false;
    for (size_t k = 0; k < lights.size(); ++k) {
        const pt_light_desc &d = s->lights[k];
        PtLight &l = lights[k];
        l.type = d.type;
        l.shadows = d.cast_shadows ? 1 : 0;
        any_shadow |= l.shadows != 0;
        std::memcpy(l.color, d.color, sizeof(l.color));
        std::memcpy(l.position, d.position, sizeof(l.position));
        // DirectionalLight / SpotLight normalise their direction at construction.
        const V3 n = vnormalize(V3{d.direction[0], d.direction[1], d.direction[2]});
        if (d.type == PT_LIGHT_POINT) {
            l.direction[0] = d.direction[0]; l.direction[1] = d.direction[1]; l.direction[2] = d.direction[2];
        } else {
            l.direction[0] = n.x; l.direction[1] = n.y; l.direction[2] = n.z;
        }
        l.radius = d.radius;
        l.half_inner = 0.5f * d.inner_angle;  // SpotLight.cpp:8
        l.half_outer = 0.5f * d.outer_angle;
    }
    // Extended estimator: emissive triangles in world space with a power CDF.
    std::vector<PtEmitter> emitters;
    std::vector<float> ecdf;
    double epower = 0.0;
    for (size_t k = 0; k < s->objects.size(); ++k) {
        const HostObject &o = s->objects[k];
        const pt_material_desc &md = s->materials[o.material];
        if (md.type != PT_MAT_EMISSIVE) continue;
        const HostTex &t = s->textures[md.tex[0]];
        double e[3] = {0, 0, 0};
        const size_t np = (size_t)t.w * t.h;
        for (size_t q = 0; q < np; ++q)
            for (int c = 0; c < 3; ++c) e[c] += t.rgba[4 * q + c];
        for (int c = 0; c < 3; ++c) e[c] /= (double)np;
        const double lum = 0.2126 * e[0] + 0.7152 * e[1] + 0.0722 * e[2];
        if (!(lum > 0.0)) continue;
        const HostMesh &m = s->meshes[o.mesh];
        auto xf = [&](uint32_t v, double out[3]) {
            const float *pp = &m.pos[3 * (size_t)v];
            for (int r2 = 0; r2 < 3; ++r2)
                out[r2] = (double)o.model[r2] * pp[0] + (double)o.model[4 + r2] * pp[1] + (double)o.model[8 + r2] * pp[2] +
                          (double)o.model[12 + r2];
        };
        for (size_t tri = 0; tri + 2 < m.idx.size(); tri += 3) {
            double a[3], b[3], c[3];
            xf(m.idx[tri], a);
            xf(m.idx[tri + 1], b);
            xf(m.idx[tri + 2], c);
            const double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, v[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
            const double cr[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
            const double area = 0.5 * std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
            if (!(area > 0.0)) continue;
            PtEmitter em;
            for (int q = 0; q < 3; ++q) {
                em.v0[q] = (float)a[q];
                em.e1[q] = (float)u[q];
                em.e2[q] = (float)v[q];
                em.emission[q] = (float)e[q];
            }
            em.lum = (float)lum;
            emitters.push_back(em);
            epower += area * lum;
            ecdf.push_back((float)epower);
        }
    }
    for (float &c : ecdf) c = (float)(c / epower);
    if (!ecdf.empty()) ecdf.back() = 1.0f;
    // Environment: piecewise-constant distribution over texels, weight = luminance x sin(theta).
    std::vector<float> efunc, emarg, econd;
    double eint = 0.0;
    uint32_t ew = 0, eh = 0;
    if (s->env_tex >= 0) {
        const HostTex &t = s->textures[(size_t)s->env_tex];
        ew = t.w;
        eh = t.h;
        efunc.resize((size_t)ew * eh);
        econd.resize((size_t)eh * (ew + 1));
        emarg.resize(eh + 1);
        std::vector<double> rows(eh);
        for (uint32_t y = 0; y < eh; ++y) {
            const double st = std::sin(3.14159265358979323846 * (y + 0.5) / eh);
            double acc = 0.0;
            econd[(size_t)y * (ew + 1)] = 0.0f;
            for (uint32_t x = 0; x < ew; ++x) {
                const float *px = &t.rgba[4 * ((size_t)y * ew + x)];
                const double f = (0.2126 * px[0] + 0.7152 * px[1] + 0.0722 * px[2]) * st * s->env_intensity;
                efunc[(size_t)y * ew + x] = (float)f;
                acc += f;
                econd[(size_t)y * (ew + 1) + x + 1] = (float)acc;
            }
            for (uint32_t x = 1; x <= ew; ++x)
                econd[(size_t)y * (ew + 1) + x] = acc > 0.0 ? (float)(econd[(size_t)y * (ew + 1) + x] / acc) : (float)x / ew;
            econd[(size_t)y * (ew + 1) + ew] = 1.0f;
            rows[y] = acc / ew;
            eint += acc;
        }
        double racc = 0.0;
        emarg[0] = 0.0f;
        for (uint32_t y = 0; y < eh; ++y) {
            racc += rows[y];
            emarg[y + 1] = (float)racc;
        }
        for (uint32_t y = 1; y <= eh; ++y) emarg[y] = racc > 0.0 ? (float)(emarg[y] / racc) : (float)y / eh;
        emarg[eh] = 1.0f;
        eint /= (double)ew * eh;  // mean over the unit square
    }
    if ((r = upload(s->d_positions, posp, st)) || (r = upload(s->d_emitters, emitters, st)) ||
        (r = upload(s->d_emitter_cdf, ecdf, st)) || (r = upload(s->d_env_func, efunc, st)) ||
        (r = upload(s->d_env_marg, emarg, st)) || (r = upload(s->d_env_cond, econd, st)))
        return r;
    if ((r = upload(s->d_meshes, meshes, st)) || (r = upload(s->d_normals, nrm, st)) || (r = upload(s->d_tangents, tan, st)) ||
        (r = upload(s->d_bitangents, bit, st)) || (r = upload(s->d_uvs, uv, st)) || (r = upload(s->d_indices, idx, st)) ||
        (r = upload(s->d_objects, objects, st)) || (r = upload(s->d_materials, mats, st)) ||
        (r = upload(s->d_tex, texd, st)) || (r = upload(s->d_texels, texels, st)) || (r = upload(s->d_lights, lights, st)))
        return r;
    RT_CUDA_TRY(cudaStreamSynchronize(st));

    PtScene &d = s->dev;
    d.nodes = s->rc->d_nodes.as<BvhNode>();
    d.tris = s->rc->d_tris.as<BvhTri>();
    d.status = s->rc->d_status.as<unsigned>();
    d.big_stack = s->rc->depth > 64 ? 1 : 0;
    d.empty = s->rc->n_tris == 0 ? 1 : 0;
    d.objects = s->d_objects.as<PtObject>();
    d.nobjects = (int)objects.size();
    d.meshes = s->d_meshes.as<PtMesh>();
    d.materials = s->d_materials.as<PtMaterial>();
    d.textures = s->d_tex.as<PtTex>();
    d.texels = s->d_texels.as<float4>();
    d.positions = s->d_positions.as<float>();
    d.normals = s->d_normals.as<float>();
    d.tangents = s->d_tangents.as<float>();
    d.bitangents = s->d_bitangents.as<float>();
    d.uvs = s->d_uvs.as<float>();
    d.indices = s->d_indices.as<uint32_t>();
    d.lights = s->d_lights.as<PtLight>();
    d.nlights = (int)lights.size();
    d.any_masked = any_masked ? 1 : 0;
    d.bg_mode = s->bg_mode;
    std::memcpy(d.bg_color, s->bg_color, sizeof(d.bg_color));
    std::memcpy(d.bg_tex, s->bg_tex, sizeof(d.bg_tex));
    (void)any_shadow;
    d.emitters = s->d_emitters.as<PtEmitter>();
    d.emitter_cdf = s->d_emitter_cdf.as<float>();
    d.nemitters = (int)emitters.size();
    d.emit_power = (float)epower;
    d.env_tex = (s->env_tex >= 0 && eint > 0.0) ? s->env_tex : -1;
    d.env_intensity = s->env_intensity;
    d.env_w = ew;
    d.env_h = eh;
    d.env_marg = s->d_env_marg.as<float>();
    d.env_cond = s->d_env_cond.as<float>();
    d.env_func = s->d_env_func.as<float>();
    d.env_integral = (float)eint;
    d.p_env = d.env_tex >= 0 ? (d.nemitters > 0 ? 0.5f : 1.0f) : 0.0f;
    // ATMOSPHERE: the caller's scattering table, or the reference's (512 x 512, 256 steps,
    // half precision) computed here.
    std::memcpy(d.sun, s->sun, sizeof(d.sun));
    d.sky = nullptr;
    d.sky_w = d.sky_h = 0;
    if (s->bg_mode == PT_BG_ATMOSPHERE) {
        const bool given = !s->sky_table.empty();
        const uint32_t w = given ? s->sky_w : kSkyTableRes, h = given ? s->sky_h : kSkyTableRes;
        if (s->d_sky.reserve((size_t)w * h * sizeof(float4)) != RT_OK) return RT_ERR_OOM;
        if (given) {
            RT_CUDA_TRY(cudaMemcpy(s->d_sky.ptr, s->sky_table.data(), s->sky_table.size() * sizeof(float),
                                   cudaMemcpyHostToDevice));
        } else {
            const int r = pt_launch_sky_table(kSkyTableRes, kSkyTableSamples, true, s->d_sky.as<float4>(), 0);
            if (r != RT_OK) return r;
            RT_CUDA_TRY(cudaDeviceSynchronize());
        }
        d.sky = s->d_sky.as<float4>();
        d.sky_w = w;
        d.sky_h = h;
    }
    s->committed = true;
    return RT_OK;
}

static int material_batch(const float *cases, size_t in_stride, const float *uniforms, size_t n, float *out,
                          size_t out_stride, int device) {
    if (!cases || !out || n >= (1ull << 31)) return arg_error("null argument or too many cases");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        set_error("CUDA device " + std::to_string(device) + " is not available");
        return RT_ERR_CUDA;
    }
    if (n == 0) return RT_OK;
    DeviceGuard g(device);
    DevBuf dc, du, dout;
    int r = RT_OK;
    if ((r = dc.reserve(n * in_stride * 4)) || (uniforms && (r = du.reserve(n * 12))) ||
        (r = dout.reserve(n * out_stride * 4))) {
        dc.release(); du.release(); dout.release();
        return r;
    }
    if (cudaMemcpy(dc.ptr, cases, n * in_stride * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        (uniforms && cudaMemcpy(du.ptr, uniforms, n * 12, cudaMemcpyHostToDevice) != cudaSuccess))
        r = RT_ERR_CUDA;
    if (r == RT_OK) r = pt_launch_material(dc.as<float>(), uniforms ? du.as<float>() : nullptr, (uint32_t)n, dout.as<float>(), 0);
    if (r == RT_OK && cudaMemcpy(out, dout.ptr, n * out_stride * 4, cudaMemcpyDeviceToHost) != cudaSuccess) r = RT_ERR_CUDA;
    if (r == RT_ERR_CUDA) set_error(std::string("material batch failed: ") + cudaGetErrorString(cudaGetLastError()));
    dc.release(); du.release(); dout.release();
    return r;
}

int pt_material_eval(const float *cases, size_t n, float *out, int device) {
    clear_error();
    return material_batch(cases, 11, nullptr, n, out, 3, device);
}

int pt_material_sample(const float *cases, const float *uniforms, size_t n, float *out, int device) {
    clear_error();
    if (!uniforms) return arg_error("null uniforms");
    return material_batch(cases, 8, uniforms, n, out, 6, device);
}

static int check_device(int device) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        set_error("CUDA device " + std::to_string(device) + " is not available");
        return RT_ERR_CUDA;
    }
    return RT_OK;
}

int pt_sky_table(uint32_t res, uint32_t samples, int32_t half_precision, float *out, int device) {
    clear_error();
    if (!out || res < 2 || res > 4096 || samples == 0) return arg_error("invalid table request");
    int r = check_device(device);
    if (r != RT_OK) return r;
    DeviceGuard g(device);
    DevBuf t;
    if ((r = t.reserve((size_t)res * res * sizeof(float4))) != RT_OK) return r;
    r = pt_launch_sky_table(res, samples, half_precision != 0, t.as<float4>(), 0);
    if (r == RT_OK && cudaMemcpy(out, t.ptr, (size_t)res * res * sizeof(float4), cudaMemcpyDeviceToHost) != cudaSuccess) {
        set_error(std::string("sky table failed: ") + cudaGetErrorString(cudaGetLastError()));
        r = RT_ERR_CUDA;
    }
    t.release();
    return r;
}

int pt_sky_eval(const float *table, uint32_t width, uint32_t height, const float *cases, size_t n, float *out,
                int device) {
    clear_error();
    if (!cases || !out || n >= (1ull << 31)) return arg_error("null argument or too many cases");
    if (table && (width == 0 || height == 0)) return arg_error("invalid table size");
    int r = check_device(device);
    if (r != RT_OK || n == 0) return r;
    DeviceGuard g(device);
    const uint32_t w = table ? width : kSkyTableRes, h = table ? height : kSkyTableRes;
    DevBuf t, dc, dout;
    if ((r = t.reserve((size_t)w * h * sizeof(float4))) || (r = dc.reserve(n * 9 * sizeof(float))) ||
        (r = dout.reserve(n * 3 * sizeof(float)))) {
        t.release(); dc.release(); dout.release();
        return r;
    }
    if (table) {
        if (cudaMemcpy(t.ptr, table, (size_t)w * h * sizeof(float4), cudaMemcpyHostToDevice) != cudaSuccess)
            r = RT_ERR_CUDA;
    } else {
        r = pt_launch_sky_table(w, kSkyTableSamples, true, t.as<float4>(), 0);
    }
    if (r == RT_OK && cudaMemcpy(dc.ptr, cases, n * 9 * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
        r = RT_ERR_CUDA;
    if (r == RT_OK) r = pt_launch_sky_eval(t.as<float4>(), w, h, dc.as<float>(), (uint32_t)n, dout.as<float>(), 0);
    if (r == RT_OK && cudaMemcpy(out, dout.ptr, n * 3 * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
        r = RT_ERR_CUDA;
    if (r == RT_ERR_CUDA) set_error(std::string("sky evaluation failed: ") + cudaGetErrorString(cudaGetLastError()));
    t.release(); dc.release(); dout.release();
    return r;
}

rt_ctx *pt_scene_raycaster(pt_scene *s) { return s ? s->rc : nullptr; }

int pt_get_render_stats(const pt_scene *s, pt_render_stats *out) {
    clear_error();
    if (!s || !out) return arg_error("null argument");
    *out = s->last;
    return RT_OK;
}

int pt_render(pt_scene *s, const pt_camera_desc *camera, uint32_t samples, uint32_t depth, uint64_t seed, float *image,
              uint32_t width, uint32_t height, uint32_t components, void *stream, uint32_t flags) {
    return pt_render_ex(s, camera, samples, depth, seed, image, width, height, components, nullptr, stream, flags);
}

// Wave capacity of a single render: 32M paths, or the largest power of two whose path state
// (about 240 bytes a path) fits in an eighth of the device's free memory -- but never less
// than the capacity the scene's engine already holds (so repeated renders keep their graph).
static uint32_t render_wave_paths(uint64_t held) {
    uint32_t cap = 1u << 25;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
        const uint64_t fit = (uint64_t)free_b / 8 / 256;
        while (cap > (1u << 20) && cap > fit) cap >>= 1;
    } else {
        cudaGetLastError();
        cap = 1u << 23;
    }
    return (uint32_t)std::min<uint64_t>(std::max<uint64_t>(cap, held), 1u << 25);
}

int pt_render_ex(pt_scene *s, const pt_camera_desc *camera, uint32_t samples, uint32_t depth, uint64_t seed,
                 float *image, uint32_t width, uint32_t height, uint32_t components, const pt_render_options *opts,
                 void *stream, uint32_t flags) {
    clear_error();
    if (!s || !camera || !image) return arg_error("null argument");
    int r = check_job(s, samples, width, height, components);
    if (r != RT_OK) return r;
    const int mode = opts ? opts->mode : PT_MODE_REFERENCE;
    if (mode != PT_MODE_REFERENCE && mode != PT_MODE_EXTENDED) return arg_error("unknown render mode");
    DeviceGuard g(s->device);
    if (!s->engine) s->engine.reset(new WaveEngine(s->device));
    const bool dev = (flags & RT_FLAG_DEVICE_PTRS) != 0;
    cudaStream_t st = dev ? static_cast<cudaStream_t>(stream) : s->rc->stream;
    JobSpec js{s,          *camera,          samples,
               depth,      seed,             image,
               width,      height,           components,
               opts ? opts->clamp : 5.0f,    opts ? opts->accum_fp64 : 0,
               opts ? opts->aov : nullptr};
    if (opts && opts->ranks > 1) {
        if (opts->rank >= opts->ranks) return arg_error("rank must be smaller than ranks");
        js.ranks = opts->ranks;
        js.rank = opts->rank;
    }
    // One tile of every pixel per wave, as many samples per wave as the wave capacity allows:
    // up to 32M paths (about 8 GB of path state and queues). Larger waves mean fewer, fuller
    // launches: the large 1080p render took 183.8 / 172.5 / 166.3 / 163.8 ms with 8M / 16M /
    // 32M / 64M paths per wave (same image).
    Tuning t{render_wave_paths(s->engine->capacity()), width * height, 1u << 30};
    if ((uint64_t)width * height > t.wave_paths) t.wave_paths = width * height;
    r = s->engine->run({js}, mode, t, dev, st, &s->last, opts && opts->profile);
    return r;
}

int pt_batch_create(pt_batch **out, int device) {
    clear_error();
    if (!out) return arg_error("null output pointer");
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        set_error("CUDA device " + std::to_string(device) + " is not available");
        return RT_ERR_CUDA;
    }
    pt_batch *b = new pt_batch();
    b->device = device;
    b->engine.reset(new WaveEngine(device));
    *out = b;
    return RT_OK;
}

int pt_batch_destroy(pt_batch *b) {
    if (!b) return RT_OK;
    DeviceGuard g(b->device);
    b->engine.reset();
    delete b;
    return RT_OK;
}

static int batch_specs(const pt_batch_job *jobs, size_t n, const pt_render_options *opts, std::vector<JobSpec> &out) {
    if (!jobs || n == 0) return arg_error("empty batch");
    out.clear();
    for (size_t k = 0; k < n; ++k) {
        const pt_batch_job &j = jobs[k];
        if (!j.scene || !j.image) return arg_error("batch job without scene or image");
        const int r = check_job(j.scene, j.samples, j.width, j.height, j.components);
        if (r != RT_OK) return r;
        out.push_back(JobSpec{j.scene, j.camera, j.samples, j.depth, j.seed, j.image, j.width, j.height, j.components,
                              opts ? opts->clamp : 5.0f, opts ? opts->accum_fp64 : 0, nullptr});
    }
    return RT_OK;
}

int pt_batch_render(pt_batch *b, const pt_batch_job *jobs, size_t n, const pt_render_options *opts,
                    const pt_batch_tuning *tuning, void *stream, uint32_t flags) {
    clear_error();
    if (!b) return arg_error("null batch");
    std::vector<JobSpec> specs;
    int r = batch_specs(jobs, n, opts, specs);
    if (r != RT_OK) return r;
    const int mode = opts ? opts->mode : PT_MODE_REFERENCE;
    if (mode != PT_MODE_REFERENCE && mode != PT_MODE_EXTENDED) return arg_error("unknown render mode");
    Tuning t = default_tuning();
    if (tuning) t = Tuning{tuning->wave_paths, tuning->tile_pixels, tuning->max_samples};
    else load_tuning(nullptr, t);
    DeviceGuard g(b->device);
    const bool dev = (flags & RT_FLAG_DEVICE_PTRS) != 0;
    return b->engine->run(specs, mode, t, dev, static_cast<cudaStream_t>(stream), &b->last, opts && opts->profile);
}

int pt_batch_get_stats(const pt_batch *b, pt_render_stats *out) {
    clear_error();
    if (!b || !out) return arg_error("null argument");
    *out = b->last;
    return RT_OK;
}

}  // extern "C"
