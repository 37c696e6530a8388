// Surface-mesh input: STL files (quest::STLReader, quest/readers/STLReader.cpp),
// the file step of signed_distance_init(file)
// (quest/interface/internal/QuestHelpers.cpp:287-320).  Host code.
//
// Format rules kept from the reference so that the same files give the same
// meshes: a file is binary when its size is exactly 84 + 50 n bytes for the
// triangle count n stored after the 80-byte header, ASCII otherwise
// (isAsciiFormat, :41-86); ASCII coordinates are the three numbers after each
// "vertex" token, parsed as C++ stream doubles (:89-126); binary coordinates
// are the nine little-endian floats of each 50-byte record widened to double
// (:129-186).  Every triangle gets its own three nodes, in file order, and
// cell i is (3i, 3i+1, 3i+2) (getMesh, :202-250).
#include "gsq_internal.cuh"

#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

namespace
{
constexpr long long STL_HEADER = 80;
constexpr long long STL_RECORD = 50;

bool host_little_endian()
{
  const uint16_t one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

template <class T>
T from_le(T v)
{
  if(host_little_endian()) return v;
  unsigned char b[sizeof(T)];
  std::memcpy(b, &v, sizeof(T));
  for(size_t i = 0; i < sizeof(T) / 2; ++i) std::swap(b[i], b[sizeof(T) - 1 - i]);
  std::memcpy(&v, b, sizeof(T));
  return v;
}

// -1: cannot open, 0: ASCII, 1: binary
int stl_kind(const char* path)
{
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if(!f.is_open()) return -1;
  f.seekg(0, std::ios::end);
  const long long size = (long long)f.tellg();
  if(size < STL_HEADER + 4) return 0;
  int32_t n = 0;
  f.seekg(STL_HEADER, std::ios::beg);
  f.read(reinterpret_cast<char*>(&n), 4);
  n = from_le(n);
  return (size == STL_HEADER + 4 + (long long)n * STL_RECORD) ? 1 : 0;
}

bool read_ascii(const char* path, std::vector<double>& nodes)
{
  std::ifstream f(path);
  if(!f.is_open()) return false;
  std::string tok;
  double x = 0.0, y = 0.0, z = 0.0;
  while(true)
  {
    // skip to the next "vertex" keyword; stop at the end of the file
    do
    {
      f >> tok;
    } while(f.good() && tok != "vertex");
    if(f.fail()) break;
    f >> x >> y >> z;
    nodes.push_back(x);
    nodes.push_back(y);
    nodes.push_back(z);
  }
  return true;
}

bool read_binary(const char* path, std::vector<double>& nodes)
{
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if(!f.is_open()) return false;
  f.seekg(STL_HEADER);
  int32_t n = 0;
  f.read(reinterpret_cast<char*>(&n), 4);
  n = from_le(n);
  nodes.reserve(9 * (size_t)std::max(n, 0));
  unsigned char rec[STL_RECORD];
  for(int32_t i = 0; i < n; ++i)
  {
    f.read(reinterpret_cast<char*>(rec), STL_RECORD);
    for(int j = 0; j < 9; ++j)  // skip the normal (3 floats); 9 vertex floats; attribute ignored
    {
      float c;
      std::memcpy(&c, rec + 12 + 4 * j, 4);
      nodes.push_back((double)from_le(c));
    }
  }
  return true;
}
}  // namespace

extern "C" {

int gsq_stl_read(const char* path, double** xyz, int32_t* nnodes, int32_t** cells, int32_t* ncells)
{
  if(!path || !xyz || !nnodes || !cells || !ncells) return gsq::fail(GSQ_ERR_INVALID, "null argument");
  *xyz = nullptr;
  *cells = nullptr;
  *nnodes = *ncells = 0;
  const int kind = stl_kind(path);
  if(kind < 0) return gsq::fail(GSQ_ERR_INVALID, std::string("cannot open the STL file ") + path);
  std::vector<double> nodes;
  if(!(kind == 1 ? read_binary(path, nodes) : read_ascii(path, nodes)))
    return gsq::fail(GSQ_ERR_INVALID, std::string("cannot read the STL file ") + path);
  const long long nn = (long long)nodes.size() / 3, nf = nn / 3;
  if(nn >= (1LL << 31) - 1) return gsq::fail(GSQ_ERR_INVALID, "STL file too large");
  auto* p = static_cast<double*>(std::malloc(sizeof(double) * std::max<size_t>(nodes.size(), 1)));
  auto* c = static_cast<int32_t*>(std::malloc(sizeof(int32_t) * 3 * std::max<long long>(nf, 1)));
  if(!p || !c)
  {
    std::free(p);
    std::free(c);
    return gsq::fail(GSQ_ERR_NOMEM, "STL arrays");
  }
  if(!nodes.empty()) std::memcpy(p, nodes.data(), sizeof(double) * nodes.size());
  for(long long i = 0; i < 3 * nf; ++i) c[i] = (int32_t)i;
  *xyz = p;
  *cells = c;
  *nnodes = (int32_t)nn;
  *ncells = (int32_t)nf;
  return GSQ_OK;
}

}  // extern "C"
