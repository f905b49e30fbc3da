// gmsh.cu — Gmsh .msh ingestion (host code): femx's GmshReader::read
// (femx/fem/GmshReader.cpp:446-548) semantics, producing the flat arrays the
// device path consumes (node-major coordinates, element-major connectivity)
// instead of a femx Mesh object.
//
// Same rules as femx: ASCII only, Gmsh 2.x and 4.x; nodes numbered in order
// of appearance; element types 1 (segment), 2 (triangle), 3 (quadrilateral),
// 4 (tetrahedron), 5 (hexahedron), 15 (point, skipped); the mesh dimension
// is the largest volume/surface element dimension; elements of that
// dimension are the mesh elements, those one dimension lower the boundary
// facets, the rest are dropped; physical tag from the element record
// (v2: first tag) or, when 0, the first physical tag of its entity (v4
// $Entities); physical names with their quotes stripped; unknown sections
// skipped. One difference: the GPU kernels take one node count per
// element, so a mesh mixing element shapes of its own dimension is
// rejected with an error. The file is read whole and tokenised in one pass.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "common.cuh"

struct gbfem_mesh
{
  int                 dim = 0;
  std::vector<double> coords; // [num_nodes][3]
  int                 nodes_per_elem  = 0;
  int                 nodes_per_facet = 0;
  std::vector<int>    conn, elem_etag, elem_ptag;
  std::vector<int>    facet_conn, facet_etag, facet_ptag;
  std::map<std::pair<int, int>, std::string> names;
};

namespace
{

using gbfem::Error;

struct Tokens
{
  std::string buf;
  size_t      p = 0;

  bool next(std::string& tok)
  {
    while (p < buf.size() && (buf[p] == ' ' || buf[p] == '\t' || buf[p] == '\n' || buf[p] == '\r'))
    {
      ++p;
    }
    if (p >= buf.size())
    {
      return false;
    }
    const size_t b = p;
    while (p < buf.size() && !(buf[p] == ' ' || buf[p] == '\t' || buf[p] == '\n' || buf[p] == '\r'))
    {
      ++p;
    }
    tok.assign(buf, b, p - b);
    return true;
  }
  std::string word()
  {
    std::string t;
    if (!next(t))
    {
      throw Error(GBFEM_EDATA, "GmshReader: unexpected end of file");
    }
    return t;
  }
  long long integer()
  {
    const std::string t = word();
    char*             end = nullptr;
    errno                 = 0;
    const long long v     = std::strtoll(t.c_str(), &end, 10);
    if (end == t.c_str() || *end != '\0' || errno != 0)
    {
      throw Error(GBFEM_EDATA, "GmshReader: expected an integer, got " + t);
    }
    return v;
  }
  double real()
  {
    const std::string t = word();
    char*             end = nullptr;
    const double      v   = std::strtod(t.c_str(), &end);
    if (end == t.c_str() || *end != '\0')
    {
      throw Error(GBFEM_EDATA, "GmshReader: expected a number, got " + t);
    }
    return v;
  }
  // rest of the current line (for $PhysicalNames)
  std::string restOfLine()
  {
    const size_t e = buf.find('\n', p);
    std::string  r = buf.substr(p, e == std::string::npos ? std::string::npos : e - p);
    p              = e == std::string::npos ? buf.size() : e + 1;
    return r;
  }
  void expect(const std::string& mark)
  {
    const std::string t = word();
    if (t != mark)
    {
      throw Error(GBFEM_EDATA, "GmshReader: expected " + mark + ", got " + t);
    }
  }
};

struct Rec
{
  int              edim = 0, etag = 0, ptag = 0, type = 0;
  std::vector<int> nids;
};

int numNodesOf(long long type)
{
  switch (type)
  {
  case 1: return 2;
  case 2: return 3;
  case 3: return 4;
  case 4: return 4;
  case 5: return 8;
  case 15: return 1;
  default:
    throw Error(GBFEM_EDATA, "GmshReader: unsupported elem type " + std::to_string(type));
  }
}

int dimOf(long long type)
{
  switch (type)
  {
  case 15: return 0;
  case 1: return 1;
  case 2:
  case 3: return 2;
  case 4:
  case 5: return 3;
  default:
    throw Error(GBFEM_EDATA, "GmshReader: unsupported elem type " + std::to_string(type));
  }
}

bool knownShape(int type)
{
  return type >= 1 && type <= 5;
}

std::string stripQuotes(const std::string& v)
{
  const size_t a = v.find('"'), b = v.rfind('"');
  if (a != std::string::npos && b != std::string::npos && a < b)
  {
    return v.substr(a + 1, b - a - 1);
  }
  return v;
}

gbfem_mesh* readGmsh(const char* path)
{
  Tokens t;
  {
    FILE* f = std::fopen(path, "rb");
    if (f == nullptr)
    {
      throw Error(GBFEM_EINVAL, std::string("GmshReader: failed to open ") + path);
    }
    char   chunk[1 << 16];
    size_t n = 0;
    while ((n = std::fread(chunk, 1, sizeof chunk, f)) > 0)
    {
      t.buf.append(chunk, n);
    }
    std::fclose(f);
  }
  double                                    version = 0.0;
  std::vector<double>                       xyz;
  std::map<long long, int>                  node_of_tag;
  std::map<std::pair<int, int>, int>        entity_ptag;
  std::map<std::pair<int, int>, std::string> names;
  std::vector<Rec>                          recs;
  std::string                               mark;
  auto node = [&](long long tag) {
    const auto it = node_of_tag.find(tag);
    if (it == node_of_tag.end())
    {
      throw Error(GBFEM_EDATA, "GmshReader: elem references unknown node " + std::to_string(tag));
    }
    return it->second;
  };
  while (t.next(mark))
  {
    if (mark == "$MeshFormat")
    {
      version             = t.real();
      const long long ft  = t.integer();
      (void) t.integer(); // data size
      if (ft != 0)
      {
        throw Error(GBFEM_EDATA, "GmshReader: only ASCII .msh files are supported");
      }
      if (!((version >= 2.0 && version < 3.0) || (version >= 4.0 && version < 5.0)))
      {
        throw Error(GBFEM_EDATA, "GmshReader: only Gmsh 2.x and 4.x .msh files are supported");
      }
      t.expect("$EndMeshFormat");
    }
    else if (mark == "$PhysicalNames")
    {
      const long long count = t.integer();
      for (long long i = 0; i < count; ++i)
      {
        const int d  = static_cast<int>(t.integer());
        const int tg = static_cast<int>(t.integer());
        names[{d, tg}] = stripQuotes(t.restOfLine());
      }
      t.expect("$EndPhysicalNames");
    }
    else if (mark == "$Entities")
    {
      long long cnt[4];
      for (auto& c : cnt)
      {
        c = t.integer();
      }
      for (int d = 0; d < 4; ++d)
      {
        for (long long i = 0; i < cnt[d]; ++i)
        {
          const int tg = static_cast<int>(t.integer());
          for (int k = 0; k < (d == 0 ? 3 : 6); ++k)
          {
            (void) t.real();
          }
          const long long np = t.integer();
          int             first = 0;
          for (long long k = 0; k < np; ++k)
          {
            const int ptag = static_cast<int>(t.integer());
            if (k == 0)
            {
              first = ptag;
            }
          }
          if (d > 0)
          {
            const long long nb = t.integer();
            for (long long k = 0; k < nb; ++k)
            {
              (void) t.integer();
            }
          }
          entity_ptag[{d, tg}] = np > 0 ? first : 0;
        }
      }
      t.expect("$EndEntities");
    }
    else if (mark == "$Nodes")
    {
      auto add = [&](long long tag, double x, double y, double z) {
        node_of_tag[tag] = static_cast<int>(xyz.size() / 3);
        xyz.push_back(x);
        xyz.push_back(y);
        xyz.push_back(z);
      };
      if (version >= 4.0)
      {
        const long long blocks = t.integer();
        (void) t.integer();
        (void) t.integer();
        (void) t.integer();
        for (long long b = 0; b < blocks; ++b)
        {
          const long long edim = t.integer();
          (void) t.integer(); // entity tag
          const long long        param = t.integer();
          const long long        nb    = t.integer();
          std::vector<long long> tags(static_cast<size_t>(nb));
          for (auto& tg : tags)
          {
            tg = t.integer();
          }
          for (long long i = 0; i < nb; ++i)
          {
            const double x = t.real(), y = t.real(), z = t.real();
            if (param)
            {
              for (long long k = 0; k < edim; ++k)
              {
                (void) t.real();
              }
            }
            add(tags[static_cast<size_t>(i)], x, y, z);
          }
        }
      }
      else
      {
        const long long n = t.integer();
        for (long long i = 0; i < n; ++i)
        {
          const long long tag = t.integer();
          const double    x = t.real(), y = t.real(), z = t.real();
          add(tag, x, y, z);
        }
      }
      t.expect("$EndNodes");
    }
    else if (mark == "$Elements")
    {
      if (version >= 4.0)
      {
        const long long blocks = t.integer();
        (void) t.integer();
        (void) t.integer();
        (void) t.integer();
        for (long long b = 0; b < blocks; ++b)
        {
          const int       edim = static_cast<int>(t.integer());
          const int       etag = static_cast<int>(t.integer());
          const int       type = static_cast<int>(t.integer());
          const long long nb   = t.integer();
          const int       nn   = numNodesOf(type);
          for (long long i = 0; i < nb; ++i)
          {
            (void) t.integer(); // element tag
            Rec r;
            r.edim = edim;
            r.etag = etag;
            r.type = type;
            for (int k = 0; k < nn; ++k)
            {
              r.nids.push_back(node(t.integer()));
            }
            if (knownShape(type))
            {
              recs.push_back(std::move(r));
            }
          }
        }
      }
      else
      {
        const long long n = t.integer();
        for (long long i = 0; i < n; ++i)
        {
          (void) t.integer(); // element tag
          const int       type = static_cast<int>(t.integer());
          const long long ntag = t.integer();
          std::vector<int> tags;
          for (long long k = 0; k < ntag; ++k)
          {
            tags.push_back(static_cast<int>(t.integer()));
          }
          const int nn = numNodesOf(type);
          Rec       r;
          r.edim = dimOf(type);
          r.ptag = ntag > 0 ? tags[0] : 0;
          r.etag = ntag > 1 ? tags[1] : 0;
          r.type = type;
          for (int k = 0; k < nn; ++k)
          {
            r.nids.push_back(node(t.integer()));
          }
          if (knownShape(type) && r.edim > 0)
          {
            recs.push_back(std::move(r));
          }
        }
      }
      t.expect("$EndElements");
    }
    else
    {
      if (mark.size() < 2 || mark[0] != '$')
      {
        throw Error(GBFEM_EDATA, "GmshReader: unexpected token " + mark);
      }
      const std::string end = "$End" + mark.substr(1);
      std::string       tok;
      bool              found = false;
      while (t.next(tok))
      {
        if (tok == end)
        {
          found = true;
          break;
        }
      }
      if (!found)
      {
        throw Error(GBFEM_EDATA, "GmshReader: missing " + end);
      }
    }
  }
  int dim = 0;
  for (const Rec& r : recs)
  {
    if (r.type == 2 || r.type == 3)
    {
      dim = dim > 2 ? dim : 2;
    }
    else if (r.type == 4 || r.type == 5)
    {
      dim = 3;
    }
  }
  if (dim == 0)
  {
    throw Error(GBFEM_EDATA, "GmshReader: no supported volume or surface elems found");
  }
  auto* m  = new gbfem_mesh;
  m->dim   = dim;
  m->coords = std::move(xyz);
  m->names  = std::move(names);
  try
  {
    for (const Rec& r : recs)
    {
      int ptag = r.ptag;
      if (ptag <= 0)
      {
        const auto it = entity_ptag.find({r.edim, r.etag});
        ptag          = it == entity_ptag.end() ? 0 : it->second;
      }
      const int nn = static_cast<int>(r.nids.size());
      if (r.edim == dim)
      {
        if (m->nodes_per_elem != 0 && m->nodes_per_elem != nn)
        {
          throw Error(GBFEM_EDATA, "GmshReader: meshes mixing element shapes are not supported");
        }
        m->nodes_per_elem = nn;
        m->conn.insert(m->conn.end(), r.nids.begin(), r.nids.end());
        m->elem_etag.push_back(r.etag);
        m->elem_ptag.push_back(ptag);
      }
      else if (r.edim == dim - 1)
      {
        if (m->nodes_per_facet != 0 && m->nodes_per_facet != nn)
        {
          throw Error(GBFEM_EDATA, "GmshReader: boundaries mixing facet shapes are not supported");
        }
        m->nodes_per_facet = nn;
        m->facet_conn.insert(m->facet_conn.end(), r.nids.begin(), r.nids.end());
        m->facet_etag.push_back(r.etag);
        m->facet_ptag.push_back(ptag);
      }
    }
  }
  catch (...)
  {
    delete m;
    throw;
  }
  return m;
}

} // namespace

extern "C" int gbfem_mesh_read_gmsh(const char* path, gbfem_mesh** out)
{
  using namespace gbfem;
  return guarded([&] {
    require(out != nullptr && path != nullptr, "GmshReader: null argument");
    *out = nullptr;
    *out = readGmsh(path);
  });
}

extern "C" int gbfem_mesh_get_view(const gbfem_mesh* m, gbfem_mesh_view* v)
{
  using namespace gbfem;
  return guarded([&] {
    require(m != nullptr && v != nullptr, "mesh handle is null");
    v->dim             = m->dim;
    v->num_nodes       = static_cast<int>(m->coords.size() / 3);
    v->num_elems       = static_cast<int>(m->elem_ptag.size());
    v->nodes_per_elem  = m->nodes_per_elem;
    v->num_facets      = static_cast<int>(m->facet_ptag.size());
    v->nodes_per_facet = m->nodes_per_facet;
    v->coords          = m->coords.data();
    v->conn            = m->conn.data();
    v->elem_etag       = m->elem_etag.data();
    v->elem_ptag       = m->elem_ptag.data();
    v->facet_conn      = m->facet_conn.data();
    v->facet_etag      = m->facet_etag.data();
    v->facet_ptag      = m->facet_ptag.data();
  });
}

extern "C" int gbfem_mesh_physical_name(const gbfem_mesh* m, int dim, int tag, char* buf,
                                        int buf_len)
{
  using namespace gbfem;
  return guarded([&] {
    require(m != nullptr && buf != nullptr && buf_len > 0, "mesh handle is null");
    const auto it = m->names.find({dim, tag});
    const std::string name = it == m->names.end() ? std::string() : it->second;
    require(static_cast<int>(name.size()) < buf_len, "physical name buffer is too small");
    std::memcpy(buf, name.c_str(), name.size() + 1);
  });
}

extern "C" void gbfem_mesh_destroy(gbfem_mesh* m)
{
  delete m;
}
