// Triangle soup mesh with the reference's interface (SimpleMesh.h:20-146):
// three fresh vertices per triangle, y negated on insertion, OFF reader and
// writer.
#pragma once

#include <algorithm>
#include <cstdint>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "kf_types.h"

typedef kf::Vec3d Vertex;

struct Triangle {
  unsigned int idx0;
  unsigned int idx1;
  unsigned int idx2;
  Triangle(unsigned int a, unsigned int b, unsigned int c) : idx0(a), idx1(b), idx2(c) {}
};

class SimpleMesh {
 public:
  SimpleMesh() {}

  // OFF reader (SimpleMesh.h:25-58).
  explicit SimpleMesh(const std::string &filepath) {
    std::ifstream in(filepath);
    if (!in.is_open()) {
      std::cout << "Failed to open " << filepath;
      return;
    }
    std::string tag;
    int nv = 0, nt = 0, ne = 0;
    in >> tag >> nv >> nt >> ne;
    m_vertices.reserve(nv);
    m_triangles.reserve(nt);
    for (int i = 0; i < nv; ++i) {
      Vertex v;
      in >> v.v[0] >> v.v[1] >> v.v[2];
      m_vertices.push_back(v);
    }
    for (int i = 0; i < nt; ++i) {
      unsigned int k, a, b, c;
      in >> k >> a >> b >> c;
      m_triangles.push_back(Triangle(a, b, c));
    }
  }

  void Clear() {
    m_vertices.clear();
    m_triangles.clear();
  }

  // SimpleMesh::AddVertex (SimpleMesh.h:66-72): y is negated.
  unsigned int AddVertex(const Vertex &vertex) {
    unsigned int id = (unsigned int)m_vertices.size();
    m_vertices.push_back(Vertex(vertex(0), -vertex(1), vertex(2)));
    return id;
  }

  unsigned int AddFace(unsigned int a, unsigned int b, unsigned int c) {
    unsigned int id = (unsigned int)m_triangles.size();
    m_triangles.push_back(Triangle(a, b, c));
    return id;
  }

  // Appends a triangle soup as produced by kf_marching_cubes (9 floats per
  // triangle, y already negated): the same vertices and faces the
  // reference's ProcessVolumeCell adds (SDF.cpp:363-375).
  void AppendSoup(const float *verts, int64_t ntri) {
    m_vertices.reserve(m_vertices.size() + 3 * ntri);
    m_triangles.reserve(m_triangles.size() + ntri);
    for (int64_t t = 0; t < ntri; ++t) {
      unsigned int base = (unsigned int)m_vertices.size();
      for (int j = 0; j < 3; ++j) {
        const float *p = verts + 9 * t + 3 * j;
        m_vertices.push_back(Vertex(p[0], p[1], p[2]));
      }
      m_triangles.push_back(Triangle(base, base + 1, base + 2));
    }
  }

  std::vector<Vertex> &GetVertices() { return m_vertices; }
  std::vector<Triangle> &GetTriangles() { return m_triangles; }

  Vertex getMinLoc() {
    Vertex r = m_vertices[0];
    for (auto &v : m_vertices)
      for (int k = 0; k < 3; ++k) r.v[k] = std::min(r.v[k], v.v[k]);
    return r;
  }
  Vertex getMaxLoc() {
    Vertex r = m_vertices[0];
    for (auto &v : m_vertices)
      for (int k = 0; k < 3; ++k) r.v[k] = std::max(r.v[k], v.v[k]);
    return r;
  }

  // OFF writer (SimpleMesh.h:113-141).
  bool WriteMesh(const std::string &filename) {
    std::ofstream out(filename);
    if (!out.is_open()) return false;
    out << "OFF" << std::endl;
    out << m_vertices.size() << " " << m_triangles.size() << " 0" << std::endl;
    for (auto &v : m_vertices) out << v.x() << " " << v.y() << " " << v.z() << std::endl;
    for (auto &t : m_triangles) out << "3 " << t.idx0 << " " << t.idx1 << " " << t.idx2 << std::endl;
    return true;
  }

 private:
  std::vector<Vertex> m_vertices;
  std::vector<Triangle> m_triangles;
};
