// The GB300 device-adapter tag (include/dax_gb300_tag.h) compiled against the
// DaxToolkit's own control headers (ArrayHandle, ArrayManagerExecution,
// Timer, the error classes): a C++ consumer of the C ABI, the way a Dax build
// selecting this tag uses it.
//
//   test_tag conformance     restates the device-adapter conformance checks
//                            of dax/cont/testing/TestingDeviceAdapter.h:
//                            ArrayManagerExecution (:290), OutOfMemory (:326),
//                            Timer (:359), the algorithms on ARRAY_SIZE 500 /
//                            OFFSET 1000 data (:919-1001, :1180-1210), and the
//                            map-cell worklet (:1093-1156, CellGradient of a
//                            linear field on a DIM^3 grid is (1,1,1))
//   test_tag cases <dir>     reads grid cases written by tests/test_tag_gpu.py
//                            (cases.txt, one name per line; <name>.in: grid,
//                            isovalue, threshold range, field), runs marching
//                            cubes (merged and not), threshold and CellGradient
//                            through the tag, and writes each output array to
//                            <name>.<output>.bin for comparison with the
//                            golden digests of the reference
//
// Exit status 0 when every check passed.
namespace dax {
namespace gb300 {
namespace cont {
struct DeviceAdapterTagGB300;
}
}  // namespace gb300
}  // namespace dax
#define DAX_DEVICE_ADAPTER DAX_DEVICE_ADAPTER_UNDEFINED
#define DAX_DEFAULT_DEVICE_ADAPTER_TAG ::dax::gb300::cont::DeviceAdapterTagGB300

#include <dax/cont/ArrayHandle.h>
#include <dax/cont/Timer.h>

#include "dax_gb300_tag.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <unistd.h>
#include <vector>

namespace {

typedef dax::gb300::cont::DeviceAdapterTagGB300 Tag;
typedef dax::cont::ArrayContainerControlTagBasic Basic;
typedef dax::cont::DeviceAdapterAlgorithm<Tag> Algorithm;
typedef dax::cont::ArrayHandle<dax::Id, Basic, Tag> IdHandle;
typedef dax::cont::ArrayHandle<dax::Scalar, Basic, Tag> ScalarHandle;
typedef dax::cont::ArrayHandle<dax::Vector3, Basic, Tag> Vector3Handle;

const dax::Id ARRAY_SIZE = 500;
const dax::Id OFFSET = 1000;
const dax::Id DIM = 8;

int g_failures = 0;

void Check(bool ok, const std::string& what) {
  if (!ok) {
    ++g_failures;
    std::cout << "FAILED: " << what << std::endl;
  }
}

template <typename T>
std::vector<T> ToHost(const dax::cont::ArrayHandle<T, Basic, Tag>& h) {
  std::vector<T> out((size_t)h.GetNumberOfValues());
  h.CopyInto(out.begin());
  return out;
}

template <typename T>
dax::cont::ArrayHandle<T, Basic, Tag> Make(const std::vector<T>& v) {
  return dax::cont::make_ArrayHandle(v, Basic(), Tag());
}

// A handle that owns its arrays: in-place algorithms refuse handles over
// user memory, so (as the reference's tests do) the values are copied into a
// new handle first.
template <typename T>
dax::cont::ArrayHandle<T, Basic, Tag> Owned(const std::vector<T>& v) {
  dax::cont::ArrayHandle<T, Basic, Tag> h;
  Algorithm::Copy(Make(v), h);
  return h;
}

void TestArrayManagerExecution() {
  std::cout << "ArrayManagerExecution" << std::endl;
  typedef dax::cont::internal::ArrayManagerExecution<dax::Scalar, Basic, Tag> Manager;
  std::vector<dax::Scalar> input((size_t)(2 * ARRAY_SIZE));
  for (dax::Id i = 0; i < 2 * ARRAY_SIZE; ++i) input[(size_t)i] = dax::Scalar(i);
  Manager manager;
  manager.LoadDataForInput(dax::cont::internal::ArrayPortalFromIterators<const dax::Scalar*>(
      input.data(), input.data() + input.size()));
  Check(manager.GetNumberOfValues() == 2 * ARRAY_SIZE, "loaded size");
  manager.Shrink(ARRAY_SIZE);
  std::vector<dax::Scalar> output((size_t)ARRAY_SIZE, -1.0f);
  manager.CopyInto(output.begin());
  for (dax::Id i = 0; i < ARRAY_SIZE; ++i)
    Check(output[(size_t)i] == dax::Scalar(i), "value copied back from the device");
  bool grew = false;
  try {
    manager.Shrink(ARRAY_SIZE + 1);
  } catch (dax::cont::ErrorControlBadValue&) {
    grew = true;
  }
  Check(grew, "Shrink refuses to grow");
  // RetrieveOutputData into a control container
  dax::cont::internal::ArrayContainerControl<dax::Scalar, Basic> container;
  manager.RetrieveOutputData(container);
  Check(container.GetNumberOfValues() == ARRAY_SIZE, "retrieved size");
  Check(container.GetPortalConst().Get(ARRAY_SIZE - 1) == dax::Scalar(ARRAY_SIZE - 1),
        "retrieved value");
}

void TestOutOfMemory() {
  std::cout << "Out of memory" << std::endl;
  // dax::Id is 32-bit, so (as in the reference test) a ridiculous size needs a
  // large element: 2^31 - 1 values of 64 scalars is 512 GiB, more than the
  // device holds; the allocation fails on the device and nothing changes.
  typedef dax::Tuple<dax::Scalar, 64> Big;
  bool got = false;
  try {
    dax::cont::internal::ArrayManagerExecution<Big, Basic, Tag> bigManager;
    dax::cont::internal::ArrayContainerControl<Big, Basic> support;
    bigManager.AllocateArrayForOutput(support, 0x7FFFFFFF);
  } catch (dax::cont::ErrorControlOutOfMemory& e) {
    got = true;
    std::cout << "  got the expected error: " << e.GetMessage() << std::endl;
  }
  Check(got, "a 512 GiB allocation reports ErrorControlOutOfMemory");
  // an allocation failure injected on the host: a limit of 1 KiB
  dax_gb300_set_alloc_limit(1024);
  got = false;
  try {
    std::vector<dax::Scalar> v(1000, 1.0f);
    ScalarHandle h = Make(v);
    h.PrepareForInput();
  } catch (dax::cont::ErrorControlOutOfMemory&) {
    got = true;
  }
  dax_gb300_set_alloc_limit(0);
  Check(got, "an injected allocation failure reports ErrorControlOutOfMemory");
  // the device still works afterwards
  std::vector<dax::Scalar> v(16, 2.0f);
  ScalarHandle h = Make(v), out;
  Algorithm::Copy(h, out);
  Check(ToHost(out) == v, "copy after an allocation failure");
}

void TestTimer() {
  std::cout << "Timer" << std::endl;
  dax::cont::Timer<Tag> timer;
  sleep(1);
  const dax::Scalar elapsed = timer.GetElapsedTime();
  std::cout << "  elapsed " << elapsed << " s" << std::endl;
  Check(elapsed > 0.999f, "Timer did not capture the full second");
  Check(elapsed < 2.0f, "Timer counted too far");
}

void TestAlgorithms() {
  std::cout << "Algorithms" << std::endl;
  // ScanInclusive / ScanExclusive of ones, returning the total
  std::vector<dax::Id> ones((size_t)ARRAY_SIZE, 1);
  IdHandle h = Make(ones), out;
  const dax::Id total = Algorithm::ScanInclusive(h, out);
  Check(total == ARRAY_SIZE, "ScanInclusive total");
  std::vector<dax::Id> s = ToHost(out);
  for (dax::Id i = 0; i < ARRAY_SIZE; ++i) Check(s[(size_t)i] == i + 1, "ScanInclusive value");
  const dax::Id etotal = Algorithm::ScanExclusive(h, out);
  Check(etotal == ARRAY_SIZE, "ScanExclusive total");
  s = ToHost(out);
  for (dax::Id i = 0; i < ARRAY_SIZE; ++i) Check(s[(size_t)i] == i, "ScanExclusive value");
  // Sort, Unique, LowerBounds / UpperBounds on i % 50 (OFFSET added)
  std::vector<dax::Id> mod((size_t)ARRAY_SIZE);
  for (dax::Id i = 0; i < ARRAY_SIZE; ++i) mod[(size_t)i] = OFFSET + (i % 50);
  IdHandle sorted = Owned(mod);
  Algorithm::Sort(sorted);
  std::vector<dax::Id> ref = mod;
  std::sort(ref.begin(), ref.end());
  Check(ToHost(sorted) == ref, "Sort");
  IdHandle uniq = Owned(ref);
  Algorithm::Unique(uniq);
  Check(uniq.GetNumberOfValues() == 50, "Unique length");
  std::vector<dax::Id> u = ToHost(uniq);
  for (dax::Id i = 0; i < 50; ++i) Check(u[(size_t)i] == OFFSET + i, "Unique value");
  IdHandle values = Make(mod), lower, upper;
  Algorithm::LowerBounds(uniq, values, lower);
  Algorithm::UpperBounds(uniq, values, upper);
  std::vector<dax::Id> lo = ToHost(lower), up = ToHost(upper);
  for (dax::Id i = 0; i < ARRAY_SIZE; ++i) {
    Check(lo[(size_t)i] == i % 50, "LowerBounds");
    Check(up[(size_t)i] == i % 50 + 1, "UpperBounds");
  }
  IdHandle inplace = Owned(mod);
  Algorithm::LowerBounds(uniq, inplace);
  Check(ToHost(inplace) == lo, "LowerBounds in place");
  // SortByKey with dax::Vector3 values
  std::vector<dax::Id> keys((size_t)ARRAY_SIZE);
  std::vector<dax::Vector3> vals((size_t)ARRAY_SIZE);
  for (dax::Id i = 0; i < ARRAY_SIZE; ++i) {
    keys[(size_t)i] = ARRAY_SIZE - 1 - i;
    vals[(size_t)i] = dax::make_Vector3(dax::Scalar(i), dax::Scalar(2 * i), dax::Scalar(3 * i));
  }
  IdHandle hk = Owned(keys);
  Vector3Handle hv = Owned(vals);
  Algorithm::SortByKey(hk, hv);
  std::vector<dax::Id> k2 = ToHost(hk);
  std::vector<dax::Vector3> v2 = ToHost(hv);
  for (dax::Id i = 0; i < ARRAY_SIZE; ++i) {
    Check(k2[(size_t)i] == i, "SortByKey keys");
    Check(v2[(size_t)i][0] == dax::Scalar(ARRAY_SIZE - 1 - i), "SortByKey values");
  }
  // StreamCompact: indices of the odd stencil entries, then those values
  std::vector<dax::Id> stencil((size_t)ARRAY_SIZE);
  std::vector<dax::Scalar> field((size_t)ARRAY_SIZE);
  for (dax::Id i = 0; i < ARRAY_SIZE; ++i) {
    stencil[(size_t)i] = i % 2;
    field[(size_t)i] = dax::Scalar(OFFSET + i);
  }
  IdHandle hs = Make(stencil), idx;
  Algorithm::StreamCompact(hs, idx);
  std::vector<dax::Id> ix = ToHost(idx);
  Check((dax::Id)ix.size() == ARRAY_SIZE / 2, "StreamCompact indices length");
  for (size_t i = 0; i < ix.size(); ++i) Check(ix[i] == dax::Id(2 * i + 1), "StreamCompact index");
  ScalarHandle hf = Make(field), kept;
  Algorithm::StreamCompact(hf, hs, kept);
  std::vector<dax::Scalar> kv = ToHost(kept);
  Check((dax::Id)kv.size() == ARRAY_SIZE / 2, "StreamCompact values length");
  for (size_t i = 0; i < kv.size(); ++i)
    Check(kv[i] == dax::Scalar(OFFSET + 2 * i + 1), "StreamCompact value");
  // Copy
  IdHandle copy;
  Algorithm::Copy(hs, copy);
  Check(ToHost(copy) == stencil, "Copy");
  // a mismatched argument is the reference's ErrorControlBadValue
  bool bad = false;
  try {
    IdHandle k3 = Owned(keys);
    Vector3Handle v3 = Owned(std::vector<dax::Vector3>(3));
    Algorithm::SortByKey(k3, v3);
  } catch (dax::cont::ErrorControlBadValue&) {
    bad = true;
  }
  Check(bad, "SortByKey with fewer values than keys is ErrorControlBadValue");
  Algorithm::Synchronize();
}

void TestWorkletMapCell() {
  std::cout << "Map cell: CellGradient" << std::endl;
  const dax_gb300_uniform_grid g = dax::gb300::cont::MakeUniformGrid(dax::Id3(DIM));
  std::vector<dax::Scalar> field((size_t)(DIM * DIM * DIM));
  for (dax::Id k = 0; k < DIM; ++k)
    for (dax::Id j = 0; j < DIM; ++j)
      for (dax::Id i = 0; i < DIM; ++i)
        field[(size_t)(i + DIM * (j + DIM * k))] = dax::Scalar(i + j + k);
  ScalarHandle hf = Make(field);
  Vector3Handle grad;
  dax::gb300::cont::CellGradient(g, hf, grad);
  std::vector<dax::Vector3> gv = ToHost(grad);
  Check((dax::Id)gv.size() == (DIM - 1) * (DIM - 1) * (DIM - 1), "one gradient per cell");
  for (size_t c = 0; c < gv.size(); ++c)
    for (int a = 0; a < 3; ++a) Check(std::fabs(gv[c][a] - 1.0f) < 1e-5f, "gradient (1,1,1)");
  // a grid the ABI refuses is the reference's ErrorControlBadValue
  bool bad = false;
  try {
    dax_gb300_uniform_grid wrong = g;
    wrong.extent_max[0] = wrong.extent_min[0] - 2;
    dax::gb300::cont::CellGradient(wrong, hf, grad);
  } catch (dax::cont::ErrorControlBadValue&) {
    bad = true;
  }
  Check(bad, "an inverted extent is ErrorControlBadValue");
}

struct CaseInput {
  dax_gb300_uniform_grid grid;
  float iso, lo, hi;
  std::vector<float> field;
};

bool ReadCase(const std::string& path, CaseInput& c) {
  std::ifstream in(path.c_str(), std::ios::binary);
  if (!in) return false;
  int32_t ext[6];
  float f[9];
  int64_t n = 0;
  in.read(reinterpret_cast<char*>(f), 6 * sizeof(float));
  in.read(reinterpret_cast<char*>(ext), 6 * sizeof(int32_t));
  in.read(reinterpret_cast<char*>(f + 6), 3 * sizeof(float));
  in.read(reinterpret_cast<char*>(&n), sizeof(n));
  for (int a = 0; a < 3; ++a) {
    c.grid.origin[a] = f[a];
    c.grid.spacing[a] = f[3 + a];
    c.grid.extent_min[a] = ext[a];
    c.grid.extent_max[a] = ext[3 + a];
  }
  c.iso = f[6];
  c.lo = f[7];
  c.hi = f[8];
  c.field.resize((size_t)n);
  in.read(reinterpret_cast<char*>(c.field.data()), n * sizeof(float));
  return (bool)in;
}

template <typename T>
void Write(const std::string& path, const std::vector<T>& v) {
  std::ofstream out(path.c_str(), std::ios::binary);
  out.write(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(T));
}

int RunCases(const std::string& dir) {
  std::ifstream list((dir + "/cases.txt").c_str());
  std::string name;
  int n = 0;
  while (list >> name) {
    CaseInput c;
    if (!ReadCase(dir + "/" + name + ".in", c)) {
      Check(false, "reading case " + name);
      continue;
    }
    ScalarHandle field = Make(c.field);
    for (int merge = 0; merge < 2; ++merge) {
      IdHandle conn;
      Vector3Handle pts;
      dax::gb300::cont::MarchingCubes(c.grid, field, c.iso, merge != 0, conn, pts);
      const std::string p = dir + "/" + name + ".mc" + std::to_string(merge);
      Write(p + ".conn.bin", ToHost(conn));
      Write(p + ".verts.bin", ToHost(pts));
    }
    IdHandle tconn;
    Vector3Handle tpts;
    ScalarHandle tfield;
    dax::gb300::cont::Threshold(c.grid, field, c.lo, c.hi, tconn, tpts, tfield);
    Write(dir + "/" + name + ".thr.conn.bin", ToHost(tconn));
    Write(dir + "/" + name + ".thr.coords.bin", ToHost(tpts));
    Write(dir + "/" + name + ".thr.field.bin", ToHost(tfield));
    Vector3Handle grad;
    dax::gb300::cont::CellGradient(c.grid, field, grad);
    Write(dir + "/" + name + ".grad.bin", ToHost(grad));
    ++n;
  }
  std::cout << n << " cases written" << std::endl;
  return n;
}

}  // namespace

int main(int argc, char** argv) {
  const std::string mode = argc > 1 ? argv[1] : "conformance";
  try {
    if (mode == "conformance") {
      TestArrayManagerExecution();
      TestOutOfMemory();
      TestTimer();
      TestAlgorithms();
      TestWorkletMapCell();
    } else if (mode == "cases" && argc > 2) {
      if (RunCases(argv[2]) == 0) Check(false, "no cases run");
    } else {
      std::cout << "usage: test_tag conformance | cases <dir>" << std::endl;
      return 2;
    }
  } catch (dax::cont::Error& e) {
    std::cout << "FAILED: uncaught " << e.GetMessage() << std::endl;
    return 1;
  }
  std::cout << (g_failures ? "FAILED " : "PASSED ") << g_failures << " failures" << std::endl;
  return g_failures ? 1 : 0;
}
