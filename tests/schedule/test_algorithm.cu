// The device adapter's generic algorithms for any type and comparison object
// (include/dax_gb300_algorithm.cuh), checked against the host's std:: versions:
// the reference suite's comparison-object cases (TestSortWithComparisonObject,
// TestLowerBounds/UpperBoundsWithComparisonObject, TestUniqueWithComparisonObject,
// dax/cont/testing/TestingDeviceAdapter.h:719-938) on its data (ARRAY_SIZE 500,
// OFFSET 1000), SortByKey with Vector3 keys and values, scans of Vector3,
// StreamCompact with a Scalar stencil, and large sorts and scans.  Built and
// run by tests/test_schedule_gpu.py; exits with the number of failures.
#include <algorithm>
#include <cstdio>
#include <numeric>
#include <random>
#include <vector>

#include "dax_gb300_algorithm.cuh"

namespace {

constexpr int ARRAY_SIZE = 500;
constexpr int OFFSET = 1000;
int failures = 0;

void check(bool ok, const char* what) {
  std::printf("%s %s\n", ok ? "PASS" : "FAIL", what);
  if (!ok) ++failures;
}

// dax::Vector3 stand-in: lexicographic order (dax::math::SortLess on tuples)
struct Vec3 {
  float x, y, z;
  __host__ __device__ Vec3() : x(0), y(0), z(0) {}
  __host__ __device__ Vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  __host__ __device__ Vec3 operator+(const Vec3& o) const { return Vec3(x + o.x, y + o.y, z + o.z); }
  __host__ __device__ bool operator<(const Vec3& o) const {
    return x < o.x || (x == o.x && (y < o.y || (y == o.y && z < o.z)));
  }
  __host__ __device__ bool operator==(const Vec3& o) const { return x == o.x && y == o.y && z == o.z; }
};

struct FuseAll {
  template <class T>
  __host__ __device__ bool operator()(const T&, const T&) const { return true; }
};

template <class T>
T* upload(const std::vector<T>& h) {
  T* d = nullptr;
  cudaMalloc(&d, sizeof(T) * (h.size() ? h.size() : 1));
  cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
  return d;
}

template <class T>
std::vector<T> fetch(const T* d, size_t n) {
  std::vector<T> h(n);
  cudaMemcpy(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost);
  return h;
}

}  // namespace

int main() {
  using namespace dax_gb300;
  std::vector<int> test(ARRAY_SIZE);
  // TestSortWithComparisonObject
  for (int i = 0; i < ARRAY_SIZE; ++i) test[i] = OFFSET + ((ARRAY_SIZE - i) % 50);
  {
    int* a = upload(test);
    int* b = upload(test);
    int st = Sort(a, ARRAY_SIZE);
    st |= Sort(b, ARRAY_SIZE, SortGreater());
    std::vector<int> sa = fetch(a, ARRAY_SIZE), sb = fetch(b, ARRAY_SIZE);
    bool ok = st == 0 && std::is_sorted(sa.begin(), sa.end());
    for (int i = 0; i < ARRAY_SIZE; ++i) ok = ok && sa[i] == sb[ARRAY_SIZE - 1 - i];
    st = Sort(b, ARRAY_SIZE, SortLess());
    ok = ok && st == 0 && fetch(b, ARRAY_SIZE) == sa;
    check(ok, "Sort with SortLess / SortGreater");
    cudaFree(a);
    cudaFree(b);
  }
  // TestLowerBounds / UpperBoundsWithComparisonObject, TestUniqueWithComparisonObject
  for (int i = 0; i < ARRAY_SIZE; ++i) test[i] = OFFSET + (i % 50);
  {
    int* input = upload(test);
    int* temp = upload(test);
    long long n = 0;
    int st = Sort(temp, ARRAY_SIZE);
    st |= Unique(temp, ARRAY_SIZE, &n);
    int32_t* out = nullptr;
    cudaMalloc(&out, sizeof(int32_t) * ARRAY_SIZE);
    st |= LowerBounds(temp, n, input, ARRAY_SIZE, out, SortLess());
    std::vector<int32_t> lo = fetch(out, ARRAY_SIZE);
    st |= UpperBounds(temp, n, input, ARRAY_SIZE, out, SortLess());
    std::vector<int32_t> up = fetch(out, ARRAY_SIZE);
    bool okl = st == 0 && n == 50, oku = okl;
    for (int i = 0; i < ARRAY_SIZE; ++i) {
      okl = okl && lo[i] == i % 50;
      oku = oku && up[i] == i % 50 + 1;
    }
    check(okl, "Unique to 50 values, then LowerBounds with SortLess");
    check(oku, "UpperBounds with SortLess");
    cudaMemcpy(temp, test.data(), sizeof(int) * ARRAY_SIZE, cudaMemcpyHostToDevice);
    st = Sort(temp, ARRAY_SIZE);
    st |= Unique(temp, ARRAY_SIZE, &n, FuseAll());
    check(st == 0 && n == 1 && fetch(temp, 1)[0] == OFFSET, "Unique with a fuse-all comparison");
    cudaFree(input);
    cudaFree(temp);
    cudaFree(out);
  }
  std::mt19937 rng(7);
  // SortByKey: Vector3 keys with int values, and int keys with Vector3 values (stable)
  {
    const int n = 20000;
    std::vector<Vec3> k(n);
    std::vector<int> v(n);
    for (int i = 0; i < n; ++i) {
      k[i] = Vec3((float)(rng() % 7), (float)(rng() % 5), (float)(rng() % 3));
      v[i] = i;
    }
    Vec3* dk = upload(k);
    int* dv = upload(v);
    int st = SortByKey(dk, dv, n);
    std::vector<int> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return k[a] < k[b]; });
    std::vector<Vec3> gk = fetch(dk, n);
    std::vector<int> gv = fetch(dv, n);
    bool ok = st == 0;
    for (int i = 0; i < n; ++i) ok = ok && gv[i] == idx[i] && gk[i] == k[idx[i]];
    check(ok, "SortByKey, Vector3 keys, stable");
    std::vector<int> ik(n);
    std::vector<Vec3> vv(n);
    for (int i = 0; i < n; ++i) {
      ik[i] = (int)(rng() % 100);
      vv[i] = Vec3((float)i, (float)-i, 0.5f);
    }
    int* dik = upload(ik);
    Vec3* dvv = upload(vv);
    st = SortByKey(dik, dvv, n, SortGreater());
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return ik[a] > ik[b]; });
    std::vector<int> gik = fetch(dik, n);
    std::vector<Vec3> gvv = fetch(dvv, n);
    ok = st == 0;
    for (int i = 0; i < n; ++i) ok = ok && gik[i] == ik[idx[i]] && gvv[i] == vv[idx[i]];
    check(ok, "SortByKey, Vector3 values, SortGreater, stable");
    cudaFree(dk);
    cudaFree(dv);
    cudaFree(dik);
    cudaFree(dvv);
  }
  // scans of Vector3 (small integers: sums are exact in float)
  {
    for (int n : {1, 1023, 1024, 1025, 300000}) {
      std::vector<Vec3> in(n);
      for (int i = 0; i < n; ++i) in[i] = Vec3((float)(i % 3), (float)(i % 5), 1.0f);
      Vec3* d = upload(in);
      Vec3* o = upload(in);
      Vec3 total;
      int st = ScanInclusive(d, o, n, &total);
      std::vector<Vec3> inc = fetch(o, n);
      st |= ScanExclusive(d, o, n);
      std::vector<Vec3> exc = fetch(o, n);
      Vec3 run;
      bool ok = st == 0;
      for (int i = 0; i < n; ++i) {
        ok = ok && exc[i] == run;
        run = run + in[i];
        ok = ok && inc[i] == run;
      }
      ok = ok && total == run;
      char what[64];
      std::snprintf(what, sizeof(what), "ScanInclusive / ScanExclusive of Vector3, n = %d", n);
      check(ok, what);
      cudaFree(d);
      cudaFree(o);
    }
  }
  // StreamCompact with a Scalar stencil
  {
    const int n = 100003;
    std::vector<long long> in(n);
    std::vector<float> sten(n);
    std::vector<long long> want;
    for (int i = 0; i < n; ++i) {
      in[i] = 3ll * i;
      sten[i] = (rng() % 3 == 0) ? 0.0f : 0.5f;
      if (sten[i] != 0.0f) want.push_back(in[i]);
    }
    long long* din = upload(in);
    float* ds = upload(sten);
    long long* dout = upload(in);
    long long m = 0;
    const int st = StreamCompact(din, ds, n, dout, &m);
    check(st == 0 && m == (long long)want.size() && fetch(dout, m) == want,
          "StreamCompact with a Scalar stencil");
    cudaFree(din);
    cudaFree(ds);
    cudaFree(dout);
  }
  // a large sort and a large scan
  {
    const int n = 1 << 21;
    std::vector<long long> h(n);
    for (int i = 0; i < n; ++i) h[i] = (long long)(rng() % 1000000) - 500000;
    long long* d = upload(h);
    const int st = Sort(d, n, SortGreater());
    std::vector<long long> want = h;
    std::stable_sort(want.begin(), want.end(), [](long long a, long long b) { return a > b; });
    check(st == 0 && fetch(d, n) == want, "Sort of 2^21 int64 with SortGreater");
    long long* o = upload(h);
    long long total = 0;
    const int st2 = ScanInclusive(d, o, n, &total);
    std::vector<long long> inc(n);
    std::partial_sum(want.begin(), want.end(), inc.begin());
    check(st2 == 0 && fetch(o, n) == inc && total == inc.back(), "ScanInclusive of 2^21 int64");
    cudaFree(d);
    cudaFree(o);
  }
  std::printf("%d failures\n", failures);
  return failures;
}
