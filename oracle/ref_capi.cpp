// C-ABI glue over the reference's OWN compiled classes -- ORACLE, test infrastructure only.
//
// Built by `make -C oracle ref` together with the reference sources compiled in place
// (Raycaster.cpp, PathTracer.cpp, MaterialGGX.cpp, ...). Nothing here restates reference
// math: every answer comes from a call into the reference code. The glue only marshals
// plain arrays into reference objects (Mesh, Object, Material, Texture, lights, Camera,
// Scene) the way the reference's loaders would fill them, and back.
//
// Used to (a) pin the C restatement in oracle/port against the reference itself and
// (b) generate the golden fixtures under tests/golden/. Only available where the
// reference tree is present; the product never links it.
#include "raycaster/Raycaster.hpp"
#include "PathTracer.hpp"
#include "MaterialGGX.hpp"
#include "MaterialSky.hpp"
#include "generation/Random.hpp"
#include "input/Camera.hpp"
#include "resources/Texture.hpp"
#include "scene/lights/DirectionalLight.hpp"
#include "scene/lights/PointLight.hpp"
#include "scene/lights/SpotLight.hpp"
#include "system/System.hpp"

#include "rendu_gb300.h"

#include <cstring>
#include <deque>
#include <memory>

Texture &shim_sky_table();  // oracle/ref_shim.cpp

namespace {

glm::mat4 to_mat4(const float *m) {
	glm::mat4 r(1.0f);
	if(m) {
		for(int c = 0; c < 4; ++c)
			for(int k = 0; k < 4; ++k) r[c][k] = m[4 * c + k];
	}
	return r;
}

struct RefRaycaster {
	Raycaster rc;
	std::deque<Mesh> meshes;
	std::vector<uint32_t> offsets; // first global triangle of each mesh
	uint32_t tris = 0;
};

void fill_hit(const RefRaycaster &r, const Raycaster::Hit &h, rt_hit &out) {
	if(!h.hit) {
		out.t	 = h.dist;
		out.u	 = 0.0f;
		out.v	 = 0.0f;
		out.prim = RT_NO_HIT;
		return;
	}
	out.t	 = h.dist;
	out.u	 = h.u;
	out.v	 = h.v;
	out.prim = r.offsets[h.meshId] + uint32_t(h.localId / 3);
}

} // namespace

extern "C" {

void *ref_rc_create() { return new RefRaycaster(); }

void ref_rc_destroy(void *h) { delete static_cast<RefRaycaster *>(h); }

// Raycaster::addMesh through a Mesh holding the given arrays.
int ref_rc_add_mesh(void *h, const float *pos, size_t nv, const uint32_t *idx, size_t ni, const float *model) {
	RefRaycaster &r = *static_cast<RefRaycaster *>(h);
	r.meshes.emplace_back("ref_mesh");
	Mesh &m = r.meshes.back();
	m.positions.resize(nv);
	for(size_t i = 0; i < nv; ++i) m.positions[i] = glm::vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
	m.indices.assign(idx, idx + ni);
	r.offsets.push_back(r.tris);
	r.tris += uint32_t(ni / 3);
	r.rc.addMesh(m, to_mat4(model));
	return int(r.offsets.size() - 1);
}

int ref_rc_build(void *h) {
	static_cast<RefRaycaster *>(h)->rc.updateHierarchy();
	return 0;
}

// rays: n x 8 floats {o.xyz, mini, d.xyz, maxi}. parallel != 0 drives the queries with the
// reference's own System::forParallel over chunks of 1024 rays.
int ref_rc_intersect(void *h, const float *rays, size_t n, rt_hit *out, int parallel) {
	const RefRaycaster &r = *static_cast<RefRaycaster *>(h);
	auto one			  = [&](size_t i) {
		 const float *q = rays + 8 * i;
		 const Raycaster::Hit hit = r.rc.intersects(glm::vec3(q[0], q[1], q[2]), glm::vec3(q[4], q[5], q[6]), q[3], q[7]);
		 fill_hit(r, hit, out[i]);
	};
	if(parallel) {
		const size_t chunk = 1024;
		System::forParallel(0, (n + chunk - 1) / chunk, [&](size_t c) {
			for(size_t i = c * chunk; i < std::min(n, (c + 1) * chunk); ++i) one(i);
		});
	} else {
		for(size_t i = 0; i < n; ++i) one(i);
	}
	return 0;
}

int ref_rc_intersect_any(void *h, const float *rays, size_t n, uint8_t *out, int parallel) {
	const RefRaycaster &r = *static_cast<RefRaycaster *>(h);
	auto one			  = [&](size_t i) {
		 const float *q = rays + 8 * i;
		 out[i] = r.rc.intersectsAny(glm::vec3(q[0], q[1], q[2]), glm::vec3(q[4], q[5], q[6]), q[3], q[7]) ? 1 : 0;
	};
	if(parallel) {
		const size_t chunk = 1024;
		System::forParallel(0, (n + chunk - 1) / chunk, [&](size_t c) {
			for(size_t i = c * chunk; i < std::min(n, (c + 1) * chunk); ++i) one(i);
		});
	} else {
		for(size_t i = 0; i < n; ++i) one(i);
	}
	return 0;
}

// Raycaster::visible on n point pairs {p0.xyz, p1.xyz}.
int ref_rc_visible(void *h, const float *segs, size_t n, uint8_t *out) {
	const RefRaycaster &r = *static_cast<RefRaycaster *>(h);
	for(size_t i = 0; i < n; ++i) {
		const float *q = segs + 6 * i;
		out[i]		   = r.rc.visible(glm::vec3(q[0], q[1], q[2]), glm::vec3(q[3], q[4], q[5])) ? 1 : 0;
	}
	return 0;
}

// ---- material model -------------------------------------------------------------------

// MaterialGGX::eval on n cases: in = n x 11 {wo.xyz, base.rgb, rough, metal, wi.xyz}.
int ref_ggx_eval(const float *in, size_t n, float *out) {
	for(size_t i = 0; i < n; ++i) {
		const float *q	 = in + 11 * i;
		const glm::vec3 r = MaterialGGX::eval(glm::vec3(q[0], q[1], q[2]), glm::vec3(q[3], q[4], q[5]), q[6], q[7],
											  glm::vec3(q[8], q[9], q[10]));
		out[3 * i + 0] = r.x;
		out[3 * i + 1] = r.y;
		out[3 * i + 2] = r.z;
	}
	return 0;
}

// MaterialGGX::sampleAndEval on n cases: in = n x 8 {wo.xyz, base.rgb, rough, metal}.
// For case i the calling thread's generator is seeded with seeds[i]; the first three
// uniforms of that stream are recorded in uniforms[3i..3i+2], the generator is re-seeded
// and sampleAndEval draws the same three numbers. out = n x 6 {weight.rgb, wi.xyz}.
int ref_ggx_sample(const float *in, const uint32_t *seeds, size_t n, float *uniforms, float *out) {
	for(size_t i = 0; i < n; ++i) {
		const float *q = in + 8 * i;
		Random::seed(seeds[i]);
		for(int k = 0; k < 3; ++k) uniforms[3 * i + k] = Random::Float();
		Random::seed(seeds[i]);
		glm::vec3 wi(0.0f);
		const glm::vec3 w = MaterialGGX::sampleAndEval(glm::vec3(q[0], q[1], q[2]), glm::vec3(q[3], q[4], q[5]), q[6], q[7], wi);
		out[6 * i + 0] = w.x;
		out[6 * i + 1] = w.y;
		out[6 * i + 2] = w.z;
		out[6 * i + 3] = wi.x;
		out[6 * i + 4] = wi.y;
		out[6 * i + 5] = wi.z;
	}
	return 0;
}

// Random::sampleCosineHemisphere after seeding: n cases, out = n x 5 {u0, u1, x, y, z}.
int ref_cosine_hemisphere(const uint32_t *seeds, size_t n, float *out) {
	for(size_t i = 0; i < n; ++i) {
		Random::seed(seeds[i]);
		out[5 * i + 0] = Random::Float();
		out[5 * i + 1] = Random::Float();
		Random::seed(seeds[i]);
		const glm::vec3 d = Random::sampleCosineHemisphere();
		out[5 * i + 2]	= d.x;
		out[5 * i + 3]	= d.y;
		out[5 * i + 4]	= d.z;
	}
	return 0;
}

// Camera::pixelShifts for a posed camera: out = {corner.xyz, dx.xyz, dy.xyz, eye.xyz}.
int ref_pixel_shifts(const pt_camera_desc *c, float *out) {
	Camera cam;
	cam.pose(glm::vec3(c->eye[0], c->eye[1], c->eye[2]), glm::vec3(c->center[0], c->center[1], c->center[2]),
			 glm::vec3(c->up[0], c->up[1], c->up[2]));
	cam.fov(c->fov);
	cam.ratio(c->ratio);
	glm::vec3 corner, dx, dy;
	cam.pixelShifts(corner, dx, dy);
	const glm::vec3 e = cam.position();
	const float v[12] = {corner.x, corner.y, corner.z, dx.x, dx.y, dx.z, dy.x, dy.y, dy.z, e.x, e.y, e.z};
	std::memcpy(out, v, sizeof(v));
	return 0;
}

// ---- path tracer -----------------------------------------------------------------------

struct RefScene {
	std::shared_ptr<Scene> scene;
	std::deque<Mesh> meshes;
	std::deque<Texture> textures;
	std::vector<pt_material_desc> matDescs;
	std::vector<std::pair<uint32_t, uint32_t>> objDescs; // (mesh, material)
	std::vector<glm::mat4> objModels;
	Material bgMaterial{Material::Type::None};
	Mesh bgMesh{"background"};
	int bgMode = PT_BG_COLOR;
	std::unique_ptr<PathTracer> tracer;
};

void *ref_pt_create() {
	RefScene *s = new RefScene();
	s->scene	= std::make_shared<Scene>("ref_scene");
	return s;
}

void ref_pt_destroy(void *h) { delete static_cast<RefScene *>(h); }

// Textures are stored as 4-channel float images (missing channels: 0, alpha 1), the
// layout Image::rgbal reads (Image.cpp:86-106).
int ref_pt_add_texture(void *h, uint32_t w, uint32_t hgt, uint32_t ch, const float *px) {
	RefScene &s = *static_cast<RefScene *>(h);
	s.textures.emplace_back("ref_tex");
	Texture &t = s.textures.back();
	t.width	= w;
	t.height   = hgt;
	t.images.emplace_back(w, hgt, 4, 0.0f);
	Image &img = t.images.back();
	for(size_t p = 0; p < size_t(w) * hgt; ++p) {
		for(uint32_t c = 0; c < 4; ++c) {
			img.pixels[4 * p + c] = c < ch ? px[ch * p + c] : (c == 3 ? 1.0f : 0.0f);
		}
	}
	return int(s.textures.size() - 1);
}

int ref_pt_add_mesh(void *h, const pt_mesh_desc *d) {
	RefScene &s = *static_cast<RefScene *>(h);
	s.meshes.emplace_back("ref_mesh");
	Mesh &m = s.meshes.back();
	auto v3 = [&](const float *a, std::vector<glm::vec3> &dst) {
		dst.resize(d->vertex_count);
		for(size_t i = 0; i < d->vertex_count; ++i) dst[i] = glm::vec3(a[3 * i], a[3 * i + 1], a[3 * i + 2]);
	};
	v3(d->positions, m.positions);
	v3(d->normals, m.normals);
	v3(d->tangents, m.tangents);
	v3(d->bitangents, m.bitangents);
	if(d->texcoords) {
		m.texcoords.resize(d->vertex_count);
		for(size_t i = 0; i < d->vertex_count; ++i) m.texcoords[i] = glm::vec2(d->texcoords[2 * i], d->texcoords[2 * i + 1]);
	}
	m.indices.assign(d->indices, d->indices + d->index_count);
	return int(s.meshes.size() - 1);
}

int ref_pt_add_material(void *h, const pt_material_desc *d) {
	RefScene &s = *static_cast<RefScene *>(h);
	s.matDescs.push_back(*d);
	return int(s.matDescs.size() - 1);
}

int ref_pt_add_object(void *h, uint32_t mesh, uint32_t material, const float *model) {
	RefScene &s = *static_cast<RefScene *>(h);
	s.objDescs.emplace_back(mesh, material);
	s.objModels.push_back(to_mat4(model));
	return int(s.objDescs.size() - 1);
}

int ref_pt_add_light(void *h, const pt_light_desc *d) {
	RefScene &s = *static_cast<RefScene *>(h);
	const glm::vec3 col(d->color[0], d->color[1], d->color[2]);
	const glm::vec3 pos(d->position[0], d->position[1], d->position[2]);
	const glm::vec3 dir(d->direction[0], d->direction[1], d->direction[2]);
	std::shared_ptr<Light> l;
	if(d->type == PT_LIGHT_POINT) {
		l = std::make_shared<PointLight>(pos, col, d->radius);
	} else if(d->type == PT_LIGHT_DIRECTIONAL) {
		l = std::make_shared<DirectionalLight>(dir, col);
	} else {
		l = std::make_shared<SpotLight>(pos, dir, col, d->inner_angle, d->outer_angle, d->radius);
	}
	l->setCastShadow(d->cast_shadows != 0);
	s.scene->lights.push_back(l);
	return 0;
}

int ref_pt_set_background(void *h, int mode, const float *color, const uint32_t *tex) {
	RefScene &s  = *static_cast<RefScene *>(h);
	s.bgMode	 = mode;
	s.bgMaterial = Material(Material::Type::None);
	if(mode == PT_BG_COLOR) {
		s.bgMaterial.addParameter(glm::vec4(color[0], color[1], color[2], 1.0f));
		s.scene->backgroundMode = Scene::Background::COLOR;
	} else if(mode == PT_BG_IMAGE) {
		s.bgMaterial.addTexture(&s.textures[tex[0]]);
		s.scene->backgroundMode = Scene::Background::IMAGE;
	} else if(mode == PT_BG_SKYBOX) {
		// A cubemap Texture with its six faces as images (+x,-x,+y,-y,+z,-z).
		s.textures.emplace_back("ref_cube");
		Texture &cube = s.textures.back();
		for(int f = 0; f < 6; ++f) {
			const Image &src = s.textures[tex[f]].images[0];
			cube.images.emplace_back(src.width, src.height, src.components, 0.0f);
			cube.images.back().pixels = src.pixels;
		}
		cube.width  = cube.images[0].width;
		cube.height = cube.images[0].height;
		s.bgMaterial.addTexture(&cube);
		s.scene->backgroundMode = Scene::Background::SKYBOX;
	} else {
		return -1;  // ATMOSPHERE needs a Sky object: its model is pinned through ref_sky_eval
	}
	return 0;
}

// PathTracer::PathTracer(scene): objects and materials are created in the given order.
int ref_pt_commit(void *h) {
	RefScene &s = *static_cast<RefScene *>(h);
	Scene &sc   = *s.scene;
	sc.materials.clear();
	sc.materials.reserve(s.matDescs.size());
	for(const pt_material_desc &d : s.matDescs) {
		sc.materials.emplace_back(Material::Type(d.type));
		Material &m = sc.materials.back();
		if(d.masked) {
			// Material::decode is the reference's only route to the masked flag.
			KeyValues kv("material");
			kv.elements.emplace_back("masked");
			kv.elements.back().values.push_back("true");
			m.decode(kv, Storage::NONE);
		}
		for(int t = 0; t < 3; ++t) m.addTexture(&s.textures[d.tex[t]]);
	}
	sc.objects.clear();
	sc.objects.reserve(s.objDescs.size());
	for(size_t o = 0; o < s.objDescs.size(); ++o) {
		sc.objects.emplace_back(&s.meshes[s.objDescs[o].first], true);
		sc.objects.back().set(s.objModels[o]);
		sc.objects.back().setMaterial(&sc.materials[s.objDescs[o].second]);
	}
	sc.background.reset(new Object(&s.bgMesh, false));
	sc.background->setMaterial(&s.bgMaterial);
	s.tracer.reset(new PathTracer(s.scene));
	return 0;
}

// PathTracer::render into a zero-initialised RGB image (w x h x 3 floats, out). The
// calling thread's generator is seeded with `seed`; render's worker threads draw their
// seeds from the shared generator, so multi-threaded renders are not reproducible.
int ref_pt_render(void *h, const pt_camera_desc *c, uint32_t spp, uint32_t depth, uint32_t seed, float *out,
				  uint32_t w, uint32_t hgt) {
	RefScene &s = *static_cast<RefScene *>(h);
	Camera cam;
	cam.pose(glm::vec3(c->eye[0], c->eye[1], c->eye[2]), glm::vec3(c->center[0], c->center[1], c->center[2]),
			 glm::vec3(c->up[0], c->up[1], c->up[2]));
	cam.fov(c->fov);
	cam.ratio(c->ratio);
	Random::seed(seed);
	Image img(w, hgt, 3, 0.0f);
	s.tracer->render(cam, spp, depth, img);
	std::memcpy(out, img.pixels.data(), sizeof(float) * size_t(w) * hgt * 3);
	return 0;
}


// Image::load (Image.cpp:108-113) of a file, as the resources manager would load it for a
// 2-D texture (no vertical flip); out receives w x h x channels floats (at most cap).
int ref_load_image(const char *path, unsigned channels, float *out, size_t cap, uint32_t *w, uint32_t *h) {
	Image img;
	const int ret = img.load(path, channels, false, true);
	if(ret != 0) return ret;
	*w = img.width;
	*h = img.height;
	const size_t n = img.pixels.size() < cap ? img.pixels.size() : cap;
	std::memcpy(out, img.pixels.data(), n * sizeof(float));
	return 0;
}

// The table MaterialSky::eval reads (w x h RGBA floats).
int ref_set_sky_table(const float *rgba, uint32_t w, uint32_t h) {
	Texture &t = shim_sky_table();
	t.images.clear();
	t.images.emplace_back(w, h, 4, 0.0f);
	std::memcpy(t.images.back().pixels.data(), rgba, sizeof(float) * 4 * size_t(w) * h);
	t.width  = w;
	t.height = h;
	return 0;
}

// MaterialSky::eval (MaterialSky.cpp:6-87) for n cases {origin, direction, sun}: n x 3 out.
int ref_sky_eval(const float *cases, size_t n, float *out) {
	for(size_t i = 0; i < n; ++i) {
		const float *c = cases + 9 * i;
		const glm::vec3 r = MaterialSky::eval(glm::vec3(c[0], c[1], c[2]), glm::vec3(c[3], c[4], c[5]),
											  glm::vec3(c[6], c[7], c[8]));
		out[3 * i]	   = r.x;
		out[3 * i + 1] = r.y;
		out[3 * i + 2] = r.z;
	}
	return 0;
}

// Image::save (Image.cpp:115-120) of w x h x c floats with the options renderOneShot uses
// (SRGB_LDR | IGNORE_ALPHA, main.cpp:119).
int ref_save_image(const float *px, uint32_t w, uint32_t h, uint32_t c, const char *path) {
	Image img(w, h, c, 0.0f);
	std::memcpy(img.pixels.data(), px, sizeof(float) * size_t(w) * h * c);
	return img.save(path, Image::Save::SRGB_LDR | Image::Save::IGNORE_ALPHA);
}
} // extern "C"
