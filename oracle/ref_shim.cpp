// Link shim for the compiled reference oracle -- ORACLE, test infrastructure only.
//
// The reference's hot-path sources (Raycaster, PathTracer, MaterialGGX, lights, Image,
// Camera, ...) compile here, but five of their neighbours cannot: Mesh.cpp, Texture.cpp,
// Codable.cpp, ResourcesManager.cpp and System.cpp include the Vulkan / windowing headers.
// This file supplies the few symbols the hot path links against from those units:
//  - trivial constructors/destructors and accessors (no computation);
//  - Codable::decodeBool and Codable::unknown, reached from Material::decode, which is the
//    reference's only route to a material's `masked` flag;
//  - Texture::sampleCubemap, the one piece of hot-path math that lives in Texture.cpp: it
//    is RESTATED here from src/engine/resources/Texture.cpp:141-191 (same face order,
//    same arithmetic) so that SKYBOX backgrounds can be rendered by the reference tracer;
//  - the resources manager reduced to what MaterialSky::eval and Image::load reach: a
//    singleton, the "scattering-precomputed" table (filled by oracle/ref_capi.cpp) and
//    plain file reads and writes (I/O only);
//  - aborting stubs for the other loaders (scene files, meshes, textures from disk), which
//    the oracle never reaches: scenes are assembled in memory by oracle/ref_capi.cpp.
#include "resources/Mesh.hpp"
#include "resources/Texture.hpp"
#include "resources/ResourcesManager.hpp"
#include "scene/Scene.hpp"
#include "system/Codable.hpp"

#include <cstdio>
#include <cstdlib>
#include <new>

class GPUMesh {};
class GPUTexture {};

[[noreturn]] static void shim_abort(const char *what) {
	std::fprintf(stderr, "reference oracle shim: %s is not available in the oracle build\n", what);
	std::abort();
}

// ---- Mesh (src/engine/resources/Mesh.cpp:96-98, 562-564, 588) --------------------------
Mesh::Mesh(const std::string &name) : _name(name) {}
Mesh::~Mesh() = default;
const std::string &Mesh::name() const { return _name; }
// The reference answers from load-time metrics; a mesh assembled in memory had texcoords
// exactly when its texcoords array is filled.
bool Mesh::hadTexcoords() const { return !texcoords.empty(); }

// ---- Texture (src/engine/resources/Texture.cpp:9-10, 96-98, 141-191) ------------------
Texture::Texture(const std::string &name) : _name(name) {}
Texture::Texture(Texture &&) = default;
Texture::~Texture() = default;

glm::vec3 Texture::sampleCubemap(const glm::vec3 &dir) const {
	// Faces in images[]: +x, -x, +y, -y, +z, -z.
	const glm::vec3 a = glm::abs(dir);
	int face		  = 0;
	float x = 0.0f, y = 0.0f, denom = 1.0f;
	if(a.x >= a.y && a.x >= a.z) {
		denom = a.x;
		y	  = dir.y;
		face  = dir.x >= 0.0f ? 0 : 1;
		x	  = dir.x >= 0.0f ? -dir.z : dir.z;
	} else if(a.y >= a.x && a.y >= a.z) {
		denom = a.y;
		x	  = dir.x;
		face  = dir.y >= 0.0f ? 2 : 3;
		y	  = dir.y >= 0.0f ? -dir.z : dir.z;
	} else if(a.z >= a.x && a.z >= a.y) {
		denom = a.z;
		y	  = dir.y;
		face  = dir.z >= 0.0f ? 4 : 5;
		x	  = dir.z >= 0.0f ? dir.x : -dir.x;
	}
	x = 0.5f * (x / denom) + 0.5f;
	y = 0.5f * (-y / denom) + 0.5f;
	// Stay one texel away from the face border.
	const float eps = 1.0f / float(std::min(images[face].width, images[face].height));
	x				= glm::clamp(x, 0.0f + eps, 1.0f - eps);
	y				= glm::clamp(y, 0.0f + eps, 1.0f - eps);
	return images[face].rgbl(x, y);
}

// ---- Scene (src/engine/scene/Scene.cpp:8-): no file is read in the oracle ------------
Scene::Scene(const std::string &) {}

// ---- Codable (src/engine/system/Codable.cpp) -----------------------------------------
bool Codable::decodeBool(const KeyValues &param, unsigned int position) {
	if(position >= param.values.size()) return false;
	const std::string &v = param.values[position];
	return v == "true" || v == "True" || v == "yes" || v == "1";
}
void Codable::unknown(const KeyValues &) {}
std::pair<std::string, Layout> Codable::decodeTexture(const KeyValues &) { shim_abort("Codable::decodeTexture"); }
glm::mat4 Codable::decodeTransformation(const std::vector<KeyValues> &) { shim_abort("Codable::decodeTransformation"); }
glm::vec2 Codable::decodeVec2(const KeyValues &, unsigned int) { shim_abort("Codable::decodeVec2"); }
glm::vec3 Codable::decodeVec3(const KeyValues &, unsigned int) { shim_abort("Codable::decodeVec3"); }
glm::vec4 Codable::decodeVec4(const KeyValues &, unsigned int) { shim_abort("Codable::decodeVec4"); }
KeyValues Codable::encode(const Texture *) { shim_abort("Codable::encode"); }
std::vector<KeyValues> Codable::encode(const glm::mat4 &) { shim_abort("Codable::encode"); }
std::string Codable::encode(bool) { shim_abort("Codable::encode"); }
std::vector<std::string> Codable::encode(const glm::vec2 &) { shim_abort("Codable::encode"); }
std::vector<std::string> Codable::encode(const glm::vec3 &) { shim_abort("Codable::encode"); }
std::vector<std::string> Codable::encode(const glm::vec4 &) { shim_abort("Codable::encode"); }

// ---- Resources (src/engine/resources/ResourcesManager.cpp) ----------------------------
// The manager is built once in static storage and never destroyed: its maps hold types
// (programs, fonts) whose destructors live in units the oracle does not compile.
Resources &Resources::manager() {
	alignas(Resources) static unsigned char storage[sizeof(Resources)];
	static Resources *instance = new(storage) Resources();
	return *instance;
}

// The sky's scattering table, served to MaterialSky::eval (MaterialSky.cpp:10).
Texture &shim_sky_table() {
	static Texture table("scattering-precomputed");
	return table;
}
const Mesh *Resources::getMesh(const std::string &, Storage) { shim_abort("Resources::getMesh"); }
char *Resources::getRawData(const std::string &, size_t &) { shim_abort("Resources::getRawData"); }
const Texture *Resources::getTexture(const std::string &name, const Layout &, Storage, const std::string &) {
	if(name == "scattering-precomputed") return &shim_sky_table();
	shim_abort("Resources::getTexture");
}
char *Resources::loadRawDataFromExternalFile(const std::string &path, size_t &size) {
	size = 0;
	FILE *f = std::fopen(path.c_str(), "rb");
	if(!f) return nullptr;
	std::fseek(f, 0, SEEK_END);
	const long len = std::ftell(f);
	std::fseek(f, 0, SEEK_SET);
	char *data = len > 0 ? static_cast<char *>(std::malloc(size_t(len))) : nullptr;
	if(data && std::fread(data, 1, size_t(len), f) == size_t(len)) {
		size = size_t(len);
	} else {
		std::free(data);
		data = nullptr;
	}
	std::fclose(f);
	return data;
}
std::string Resources::loadStringFromExternalFile(const std::string &) {
	shim_abort("Resources::loadStringFromExternalFile");
}
void Resources::saveRawDataToExternalFile(const std::string &path, char *data, size_t size) {
	FILE *f = std::fopen(path.c_str(), "wb");
	if(!f) return;
	std::fwrite(data, 1, size, f);
	std::fclose(f);
}
