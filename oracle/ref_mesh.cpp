// ORACLE, test infrastructure only: the mesh loading of the reference's offline renderer
// (Resources::getMesh with Storage::CPU | Storage::FORCE_FRAME, ResourcesManager.cpp:306-340
// of kosua20/Rendu), used to pin rendu_gb300/meshio.py.
//
// Mesh.cpp itself includes the Vulkan headers and does not compile in this tree, so its three
// steps are written out here with the reference's own building blocks:
//   * the OBJ Indexed loader (Mesh.cpp:99-271) with the C++ library calls the reference
//     makes (std::getline, stringstream token split, std::stof / std::stoi, substr with the
//     reference's count arguments);
//   * computeNormals (Mesh.cpp:327-354) with the reference's glm;
//   * computeTangentsAndBitangents (Mesh.cpp:356-505): the reference's OWN copy of
//     mikktspace.c (src/libs/mikktspace, compiled in place) behind callbacks that read the
//     mesh as Mesh.cpp:25-92 do, then the vertex split and the tangent finish with glm.
#include <glm/glm.hpp>
#include <glm/gtc/matrix_transform.hpp>
#include <mikktspace/mikktspace.h>

#include <cstdint>
#include <cstring>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

struct LoadedMesh {
	std::vector<glm::vec3> positions, normals, tangents, bitangents;
	std::vector<glm::vec2> texcoords;
	std::vector<uint32_t> indices;
	bool had_uv = false;
};

LoadedMesh g_mesh;
std::string g_error;

std::string trim_cr(const std::string &s) {
	size_t a = 0, b = s.size();
	while(a < b && s[a] == '\r') ++a;
	while(b > a && s[b - 1] == '\r') --b;
	return s.substr(a, b - a);
}

// Mesh.cpp:99-271, Load::Indexed.
bool parse_obj(const std::string &text, LoadedMesh &m) {
	std::vector<glm::vec3> pos_t, nor_t;
	std::vector<glm::vec2> uv_t;
	std::vector<std::string> faces;
	std::stringstream in(text);
	std::string line;
	while(!in.eof()) {
		std::getline(in, line);
		if(line.empty() || line[0] == '#' || line.size() < 2) continue;
		std::stringstream ss(trim_cr(line));
		std::vector<std::string> tok;
		std::string t;
		while(ss >> t) tok.push_back(t);
		if(tok.empty()) continue;
		if(tok[0] == "v" && tok.size() >= 4) {
			pos_t.emplace_back(std::stof(tok[1]), std::stof(tok[2]), std::stof(tok[3]));
		} else if(tok[0] == "vn" && tok.size() >= 4) {
			nor_t.emplace_back(std::stof(tok[1]), std::stof(tok[2]), std::stof(tok[3]));
		} else if(tok[0] == "vt" && tok.size() >= 3) {
			uv_t.emplace_back(std::stof(tok[1]), 1.0f - std::stof(tok[2]));
		} else if(tok[0] == "f" && tok.size() >= 4) {
			faces.push_back(tok[1]);
			faces.push_back(tok[2]);
			faces.push_back(tok[3]);
		}
	}
	if(pos_t.empty()) return true;
	const bool has_uv = !uv_t.empty(), has_n = !nor_t.empty();
	std::unordered_map<std::string, uint32_t> seen;
	uint32_t next = 0;
	for(const std::string &s : faces) {
		auto it = seen.find(s);
		if(it != seen.end()) {
			m.indices.push_back(it->second);
			continue;
		}
		const size_t first = s.find_first_of('/');
		const size_t last  = s.find_last_of('/');
		const long p	   = long(std::stoi(s.substr(0, first))) - 1;
		if(p < 0 || p >= (long)pos_t.size()) {
			g_error = "position index out of range";
			return false;
		}
		m.positions.push_back(pos_t[p]);
		if(has_uv) {
			const long u = long(std::stoi(s.substr(first + 1, last))) - 1;
			if(u < 0 || u >= (long)uv_t.size()) {
				g_error = "texcoord index out of range";
				return false;
			}
			m.texcoords.push_back(uv_t[u]);
		}
		if(has_n) {
			const long n = long(std::stoi(s.substr(last + 1))) - 1;
			if(n < 0 || n >= (long)nor_t.size()) {
				g_error = "normal index out of range";
				return false;
			}
			m.normals.push_back(nor_t[n]);
		}
		m.indices.push_back(next);
		seen[s] = next++;
	}
	m.had_uv = has_uv;
	return true;
}

// Mesh.cpp:327-354.
void compute_normals(LoadedMesh &m) {
	m.normals.assign(m.positions.size(), glm::vec3(0.0f));
	for(size_t t = 0; t + 2 < m.indices.size(); t += 3) {
		const uint32_t i0 = m.indices[t], i1 = m.indices[t + 1], i2 = m.indices[t + 2];
		const glm::vec3 a = glm::normalize(m.positions[i1] - m.positions[i0]);
		const glm::vec3 b = glm::normalize(m.positions[i2] - m.positions[i0]);
		const glm::vec3 n = glm::cross(a, b);
		m.normals[i0] += n;
		m.normals[i1] += n;
		m.normals[i2] += n;
	}
	for(auto &n : m.normals) n = glm::normalize(n);
}

// MikkTSpace callbacks reading the mesh per face corner (Mesh.cpp:25-92).
struct MikkData {
	const LoadedMesh *mesh;
	std::vector<glm::vec4> corner;
};
int mk_faces(const SMikkTSpaceContext *c) { return int(((MikkData *)c->m_pUserData)->mesh->indices.size() / 3); }
int mk_verts(const SMikkTSpaceContext *, const int) { return 3; }
void mk_pos(const SMikkTSpaceContext *c, float out[], const int f, const int v) {
	const LoadedMesh &m = *((MikkData *)c->m_pUserData)->mesh;
	const glm::vec3 &p	= m.positions[m.indices[3 * f + v]];
	out[0] = p.x, out[1] = p.y, out[2] = p.z;
}
void mk_nor(const SMikkTSpaceContext *c, float out[], const int f, const int v) {
	const LoadedMesh &m = *((MikkData *)c->m_pUserData)->mesh;
	const glm::vec3 &n	= m.normals[m.indices[3 * f + v]];
	out[0] = n.x, out[1] = n.y, out[2] = n.z;
}
void mk_uv(const SMikkTSpaceContext *c, float out[], const int f, const int v) {
	const LoadedMesh &m = *((MikkData *)c->m_pUserData)->mesh;
	const glm::vec2 &u	= m.texcoords[m.indices[3 * f + v]];
	out[0] = u.x, out[1] = u.y;
}
void mk_set(const SMikkTSpaceContext *c, const float t[], const float sign, const int f, const int v) {
	((MikkData *)c->m_pUserData)->corner[3 * f + v] = glm::vec4(t[0], t[1], t[2], sign);
}

bool run_mikktspace(const LoadedMesh &m, std::vector<glm::vec4> &corner) {
	SMikkTSpaceInterface itf;
	std::memset(&itf, 0, sizeof(itf));
	itf.m_getNumFaces		   = mk_faces;
	itf.m_getNumVerticesOfFace = mk_verts;
	itf.m_getPosition		   = mk_pos;
	itf.m_getNormal			   = mk_nor;
	itf.m_getTexCoord		   = mk_uv;
	itf.m_setTSpaceBasic	   = mk_set;
	MikkData data{&m, std::vector<glm::vec4>(m.indices.size())};
	SMikkTSpaceContext ctx;
	ctx.m_pInterface = &itf;
	ctx.m_pUserData	 = &data;
	const bool ok	 = genTangSpaceDefault(&ctx) != 0;
	corner			 = std::move(data.corner);
	return ok;
}

// Mesh.cpp:356-505 with force = true.
void compute_frames(LoadedMesh &m) {
	if(m.positions.empty() || m.normals.empty()) return;
	if(m.texcoords.empty()) m.texcoords.assign(m.positions.size(), glm::vec2(0.5f));
	std::vector<glm::vec4> corner;
	if(!run_mikktspace(m, corner)) {
		m.tangents.assign(m.positions.size(), glm::vec3(1.0f, 0.0f, 0.0f));
		m.bitangents.assign(m.positions.size(), glm::vec3(0.0f, 1.0f, 0.0f));
		return;
	}
	const size_t nv = m.positions.size();
	std::vector<std::vector<uint32_t>> inst(nv);  // corners of each vertex, increasing
	for(uint32_t c = 0; c < m.indices.size(); ++c) inst[m.indices[c]].push_back(c);
	// split: an instance whose tangent differs from the previous instance's gets a new vertex
	std::vector<int64_t> new_slot(m.indices.size(), -1);
	std::vector<uint32_t> extra_vertex, extra_corner;
	for(uint32_t v = 0; v < nv; ++v)
		for(size_t r = 1; r < inst[v].size(); ++r)
			if(!(corner[inst[v][r]] == corner[inst[v][r - 1]])) {
				new_slot[inst[v][r]] = int64_t(nv + extra_vertex.size());
				extra_vertex.push_back(v);
				extra_corner.push_back(inst[v][r]);
			}
	const size_t total = nv + extra_vertex.size();
	m.positions.resize(total);
	m.normals.resize(total);
	m.texcoords.resize(total);
	m.tangents.resize(total);
	m.bitangents.resize(total);
	auto finish = [&](uint32_t c, size_t v) {
		const glm::vec4 &tg = corner[c];
		glm::vec3 t			= glm::vec3(tg);
		if(glm::length(glm::cross(m.normals[v], t)) < 0.01f)
			t = std::abs(m.normals[v].z) > 0.01f ? glm::vec3(1.0f, 0.0f, 0.0f) : glm::vec3(0.0f, 0.0f, 1.0f);
		m.bitangents[v] = glm::normalize(-tg.w * glm::cross(m.normals[v], t));
		m.tangents[v]	= glm::normalize(t);
	};
	for(uint32_t v = 0; v < nv; ++v) {
		if(inst[v].empty()) continue;
		finish(inst[v][0], v);
		for(size_t r = 1; r < inst[v].size(); ++r) {
			const uint32_t c = inst[v][r];
			if(new_slot[c] < 0) {
				m.indices[c] = m.indices[inst[v][r - 1]];
				continue;
			}
			const size_t dst = size_t(new_slot[c]);
			m.indices[c]	 = uint32_t(dst);
			m.positions[dst] = m.positions[v];
			m.normals[dst]	 = m.normals[v];
			m.texcoords[dst] = m.texcoords[v];
			finish(c, dst);
		}
	}
}

template <typename T>
void copy_out(const std::vector<T> &v, float *dst) {
	if(dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(T));
}

} // namespace

extern "C" {

// Load an OBJ text as getMesh(FORCE_FRAME) does. counts = {vertices, indices, had_uv}.
int ref_mesh_load_obj(const char *text, size_t len, uint64_t *counts) {
	g_mesh = LoadedMesh();
	g_error.clear();
	try {
		if(!parse_obj(std::string(text, len), g_mesh)) return 1;
	} catch(const std::exception &e) {
		g_error = e.what();
		return 2;
	}
	if(g_mesh.normals.empty()) compute_normals(g_mesh);
	compute_frames(g_mesh);
	counts[0] = g_mesh.positions.size();
	counts[1] = g_mesh.indices.size();
	counts[2] = g_mesh.had_uv ? 1 : 0;
	return 0;
}

const char *ref_mesh_error() { return g_error.c_str(); }

// The arrays of the last ref_mesh_load_obj (sizes from its counts).
int ref_mesh_get(float *pos, float *nor, float *uv, float *tan, float *bit, uint32_t *idx) {
	copy_out(g_mesh.positions, pos);
	copy_out(g_mesh.normals, nor);
	copy_out(g_mesh.texcoords, uv);
	copy_out(g_mesh.tangents, tan);
	copy_out(g_mesh.bitangents, bit);
	if(idx && !g_mesh.indices.empty()) std::memcpy(idx, g_mesh.indices.data(), g_mesh.indices.size() * 4);
	return 0;
}

// The reference's mikktspace.c on a triangle list: per-corner (tangent, sign), 4 floats each.
int ref_mikktspace(const float *pos, const float *nor, const float *uv, size_t nv, const uint32_t *idx, size_t ni,
				   float *out) {
	LoadedMesh m;
	m.positions.assign((const glm::vec3 *)pos, (const glm::vec3 *)pos + nv);
	m.normals.assign((const glm::vec3 *)nor, (const glm::vec3 *)nor + nv);
	m.texcoords.assign((const glm::vec2 *)uv, (const glm::vec2 *)uv + nv);
	m.indices.assign(idx, idx + ni);
	std::vector<glm::vec4> corner;
	if(!run_mikktspace(m, corner)) return 1;
	std::memcpy(out, corner.data(), corner.size() * sizeof(glm::vec4));
	return 0;
}

// Codable::decodeTransformation's matrix (Codable.cpp:79-104) from decoded values, with the
// reference's glm: translate * rotate(angle, normalize(axis)) * scale; column-major out.
int ref_transformation(const float *axis, float angle, const float *trans, float scale, float *out) {
	glm::vec3 a(axis[0], axis[1], axis[2]);
	a						 = glm::normalize(a);
	const glm::mat4 t		 = glm::translate(glm::mat4(1.0f), glm::vec3(trans[0], trans[1], trans[2]));
	const glm::mat4 r		 = angle != 0.0f ? glm::rotate(glm::mat4(1.0f), angle, a) : glm::mat4(1.0f);
	const glm::mat4 s		 = glm::scale(glm::mat4(1.0f), glm::vec3(scale));
	const glm::mat4 m		 = t * r * s;
	std::memcpy(out, &m[0][0], 16 * sizeof(float));
	return 0;
}

// glm's mat4 product a * b (column-major in and out).
int ref_mat_mul(const float *a, const float *b, float *out) {
	glm::mat4 ma, mb;
	std::memcpy(&ma[0][0], a, 16 * sizeof(float));
	std::memcpy(&mb[0][0], b, 16 * sizeof(float));
	const glm::mat4 m = ma * mb;
	std::memcpy(out, &m[0][0], 16 * sizeof(float));
	return 0;
}

} // extern "C"
