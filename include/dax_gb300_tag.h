// The GB300 device adapter for the DaxToolkit control environment.
//
// A Dax build selects a device adapter by a tag type for which the
// reference's templates are specialised (dax/cont/internal/DeviceAdapterTag.h:
// 22-79; with DAX_DEVICE_ADAPTER set to DAX_DEVICE_ADAPTER_UNDEFINED and
// DAX_DEFAULT_DEVICE_ADAPTER_TAG to ::dax::gb300::cont::DeviceAdapterTagGB300,
// this tag becomes the default).  This header is that tag, on the C ABI of
// dax_gb300.h:
//
//   * dax::gb300::cont::DeviceAdapterTagGB300;
//   * ArrayManagerExecution<T, ArrayContainerControlTagBasic, TagGB300>
//     (dax/cont/internal/ArrayManagerExecution.h:44-143): device arrays,
//     allocated and copied through dax_gb300_device_alloc / dax_gb300_memcpy;
//     portals are dax::exec::internal::ArrayPortalFromIterators over device
//     pointers;
//   * DeviceAdapterTimerImplementation<TagGB300>
//     (dax/cont/internal/DeviceAdapterAlgorithm.h:343-406): device events;
//   * DeviceAdapterAlgorithm<TagGB300> (DeviceAdapterAlgorithm.h:44-331):
//     Copy, LowerBounds, UpperBounds, ScanInclusive, ScanExclusive, Sort,
//     SortByKey, StreamCompact, Unique and Synchronize for the element types
//     the C ABI sorts and scans (dax::Id, dax::Scalar, 32/64-bit integers;
//     sort and compaction values of 4, 8, 12 or 16 bytes, such as
//     dax::Vector3).  Schedule and the comparison-object forms run device
//     code and come from dax_gb300_schedule.cuh / dax_gb300_algorithm.cuh
//     in a CUDA translation unit;
//   * the hot-path dispatch behind DispatcherMapCell<MarchingCubesCount |
//     ThresholdCount | CellGradient> and the generate dispatchers on a uniform
//     grid (dax::gb300::cont::MarchingCubes, Threshold, CellGradient): the
//     calls a dispatcher specialisation for this tag makes.
//
// Status codes become the reference's exceptions: BAD_VALUE, CAPACITY and
// UNSUPPORTED ErrorControlBadValue, OUT_OF_MEMORY ErrorControlOutOfMemory,
// everything raised on the device or by CUDA ErrorExecution.  All calls are
// on the default stream and synchronous where the reference returns a value
// to the host, as the reference's CUDA adapter is.
//
// Include after the Dax headers are on the include path; compile as C++11.
#ifndef DAX_GB300_TAG_H
#define DAX_GB300_TAG_H

#include <dax/Types.h>
#include <dax/cont/ArrayContainerControlBasic.h>
#include <dax/cont/ArrayHandle.h>
#include <dax/cont/ErrorControlBadValue.h>
#include <dax/cont/ErrorControlOutOfMemory.h>
#include <dax/cont/ErrorExecution.h>
#include <dax/cont/internal/ArrayManagerExecution.h>
#include <dax/cont/internal/DeviceAdapterAlgorithm.h>
#include <dax/exec/internal/ArrayPortalFromIterators.h>

#include <cstdint>
#include <limits>
#include <string>
#include <vector>

#include "dax_gb300.h"

namespace dax {
namespace gb300 {
namespace cont {

/// The device-adapter tag of the GB300 adapter.
struct DeviceAdapterTagGB300 {};

namespace internal {

/// Throws the reference's exception for a non-zero C-ABI status.
inline void Check(int status) {
  if (status == DAX_GB300_SUCCESS) return;
  const std::string msg = dax_gb300_last_error();
  switch (status) {
    case DAX_GB300_ERROR_BAD_VALUE:
    case DAX_GB300_ERROR_CAPACITY:
    case DAX_GB300_ERROR_UNSUPPORTED:
      throw dax::cont::ErrorControlBadValue(msg);
    case DAX_GB300_ERROR_OUT_OF_MEMORY:
      throw dax::cont::ErrorControlOutOfMemory(msg);
    default:
      throw dax::cont::ErrorExecution(msg);
  }
}

/// Bytes of n values of T, or an out-of-memory error when that overflows.
template <typename T>
inline uint64_t ByteSize(dax::Id n) {
  if (n < 0) throw dax::cont::ErrorControlBadValue("negative array size");
  if ((uint64_t)n > std::numeric_limits<uint64_t>::max() / sizeof(T))
    throw dax::cont::ErrorControlOutOfMemory("array size overflows the address space");
  return (uint64_t)n * sizeof(T);
}

/// A device buffer owned by the host (scratch of one algorithm call).
class DeviceBuffer {
 public:
  explicit DeviceBuffer(uint64_t bytes) { Check(dax_gb300_device_alloc(&this->Ptr, bytes)); }
  ~DeviceBuffer() { dax_gb300_device_free(this->Ptr); }
  void* Get() const { return this->Ptr; }

 private:
  DeviceBuffer(const DeviceBuffer&);
  DeviceBuffer& operator=(const DeviceBuffer&);
  void* Ptr = nullptr;
};

/// C-ABI element type code of T (-1: not a C-ABI key type).
template <typename T> struct TypeCode { static const int value = -1; };
template <> struct TypeCode<int32_t> { static const int value = DAX_GB300_TYPE_I32; };
template <> struct TypeCode<uint32_t> { static const int value = DAX_GB300_TYPE_U32; };
template <> struct TypeCode<float> { static const int value = DAX_GB300_TYPE_F32; };
template <> struct TypeCode<int64_t> { static const int value = DAX_GB300_TYPE_I64; };
template <> struct TypeCode<uint64_t> { static const int value = DAX_GB300_TYPE_U64; };

template <typename T>
inline int KeyType() {
  static_assert(TypeCode<T>::value >= 0,
                "this algorithm runs on dax::Id, dax::Scalar and 32/64-bit integer keys; use "
                "dax_gb300_algorithm.cuh for other types");
  return TypeCode<T>::value;
}

}  // namespace internal
}  // namespace cont
}  // namespace gb300
}  // namespace dax

namespace dax {
namespace cont {
namespace internal {

/// ArrayManagerExecution for the GB300 tag: the execution array is device
/// memory of this library's allocator, the control array a basic container.
template <typename T>
class ArrayManagerExecution<T, dax::cont::ArrayContainerControlTagBasic,
                            dax::gb300::cont::DeviceAdapterTagGB300> {
 public:
  typedef T ValueType;
  typedef dax::exec::internal::ArrayPortalFromIterators<ValueType*> PortalType;
  typedef dax::exec::internal::ArrayPortalFromIterators<const ValueType*> PortalConstType;
  typedef dax::cont::internal::ArrayContainerControl<T, dax::cont::ArrayContainerControlTagBasic>
      ContainerType;

  ArrayManagerExecution() : Array(nullptr), NumberOfValues(0), AllocatedValues(0) {}
  ~ArrayManagerExecution() { this->ReleaseResources(); }

  dax::Id GetNumberOfValues() const { return this->NumberOfValues; }

  void LoadDataForInput(typename ContainerType::PortalConstType portal) {
    this->Allocate(portal.GetNumberOfValues());
    this->ToDevice(portal.GetIteratorBegin(), this->NumberOfValues);
  }

  void LoadDataForInPlace(typename ContainerType::PortalType portal) {
    this->LoadDataForInput(typename ContainerType::PortalConstType(portal));
  }

  void AllocateArrayForOutput(ContainerType&, dax::Id numberOfValues) {
    this->Allocate(numberOfValues);
  }

  void RetrieveOutputData(ContainerType& controlArray) const {
    controlArray.Allocate(this->NumberOfValues);
    this->CopyInto(controlArray.GetPortal().GetIteratorBegin());
  }

  template <class IteratorTypeControl>
  void CopyInto(IteratorTypeControl dest) const {
    std::vector<T> host((size_t)this->NumberOfValues);
    if (this->NumberOfValues > 0)
      dax::gb300::cont::internal::Check(
          dax_gb300_memcpy(host.data(), this->Array,
                           dax::gb300::cont::internal::ByteSize<T>(this->NumberOfValues),
                           DAX_GB300_DEVICE_TO_HOST));
    for (dax::Id i = 0; i < this->NumberOfValues; ++i, ++dest) *dest = host[(size_t)i];
  }

  void Shrink(dax::Id numberOfValues) {
    if (numberOfValues > this->NumberOfValues)
      throw dax::cont::ErrorControlBadValue("Shrink method cannot be used to grow array.");
    this->NumberOfValues = numberOfValues;
  }

  PortalType GetPortal() {
    return PortalType(this->Array, this->Array + this->NumberOfValues);
  }
  PortalConstType GetPortalConst() const {
    return PortalConstType(this->Array, this->Array + this->NumberOfValues);
  }

  void ReleaseResources() {
    if (this->Array) dax_gb300_device_free(this->Array);
    this->Array = nullptr;
    this->NumberOfValues = this->AllocatedValues = 0;
  }

 private:
  ArrayManagerExecution(const ArrayManagerExecution&);
  void operator=(const ArrayManagerExecution&);

  void Allocate(dax::Id n) {
    if (n <= this->AllocatedValues) {
      this->NumberOfValues = n;
      return;
    }
    const uint64_t bytes = dax::gb300::cont::internal::ByteSize<T>(n);
    this->ReleaseResources();
    void* p = nullptr;
    dax::gb300::cont::internal::Check(dax_gb300_device_alloc(&p, bytes));
    this->Array = static_cast<T*>(p);
    this->NumberOfValues = this->AllocatedValues = n;
  }

  template <typename It>
  void ToDevice(It begin, dax::Id n) {
    if (n <= 0) return;
    std::vector<T> host(begin, begin + n);
    dax::gb300::cont::internal::Check(dax_gb300_memcpy(
        this->Array, host.data(), dax::gb300::cont::internal::ByteSize<T>(n),
        DAX_GB300_HOST_TO_DEVICE));
  }

  T* Array;
  dax::Id NumberOfValues;
  dax::Id AllocatedValues;
};

}  // namespace internal

/// dax::cont::Timer<DeviceAdapterTagGB300>: device events around the timed
/// work (wall time between Reset and GetElapsedTime, all queued work
/// finished).
template <>
class DeviceAdapterTimerImplementation<dax::gb300::cont::DeviceAdapterTagGB300> {
 public:
  DeviceAdapterTimerImplementation() : Timer(nullptr) {
    dax::gb300::cont::internal::Check(dax_gb300_timer_create(&this->Timer));
    this->Reset();
  }
  ~DeviceAdapterTimerImplementation() { dax_gb300_timer_destroy(this->Timer); }

  void Reset() {
    dax::gb300::cont::internal::Check(dax_gb300_synchronize(nullptr));
    dax::gb300::cont::internal::Check(dax_gb300_timer_start(this->Timer, nullptr));
  }

  dax::Scalar GetElapsedTime() {
    double s = 0.0;
    dax::gb300::cont::internal::Check(dax_gb300_timer_elapsed(this->Timer, nullptr, &s));
    return dax::Scalar(s);
  }

 private:
  DeviceAdapterTimerImplementation(const DeviceAdapterTimerImplementation&);
  void operator=(const DeviceAdapterTimerImplementation&);
  void* Timer;
};

/// The device-adapter algorithms of the GB300 tag, on the C ABI.
template <>
struct DeviceAdapterAlgorithm<dax::gb300::cont::DeviceAdapterTagGB300> {
  typedef dax::gb300::cont::DeviceAdapterTagGB300 Tag;

  template <typename T, class CIn, class COut>
  static void Copy(const dax::cont::ArrayHandle<T, CIn, Tag>& input,
                   dax::cont::ArrayHandle<T, COut, Tag>& output) {
    const dax::Id n = input.GetNumberOfValues();
    const T* in = input.PrepareForInput().GetIteratorBegin();
    T* out = output.PrepareForOutput(n).GetIteratorBegin();
    dax::gb300::cont::internal::Check(dax_gb300_memcpy(
        out, in, dax::gb300::cont::internal::ByteSize<T>(n), DAX_GB300_DEVICE_TO_DEVICE));
  }

  template <typename T, class CIn, class CVal, class COut>
  static void LowerBounds(const dax::cont::ArrayHandle<T, CIn, Tag>& input,
                          const dax::cont::ArrayHandle<T, CVal, Tag>& values,
                          dax::cont::ArrayHandle<dax::Id, COut, Tag>& output) {
    Bounds(input, values, output, 0);
  }
  template <class CIn, class COut>
  static void LowerBounds(const dax::cont::ArrayHandle<dax::Id, CIn, Tag>& input,
                          dax::cont::ArrayHandle<dax::Id, COut, Tag>& values_output) {
    BoundsInPlace(input, values_output, 0);
  }
  template <typename T, class CIn, class CVal, class COut>
  static void UpperBounds(const dax::cont::ArrayHandle<T, CIn, Tag>& input,
                          const dax::cont::ArrayHandle<T, CVal, Tag>& values,
                          dax::cont::ArrayHandle<dax::Id, COut, Tag>& output) {
    Bounds(input, values, output, 1);
  }
  template <class CIn, class COut>
  static void UpperBounds(const dax::cont::ArrayHandle<dax::Id, CIn, Tag>& input,
                          dax::cont::ArrayHandle<dax::Id, COut, Tag>& values_output) {
    BoundsInPlace(input, values_output, 1);
  }

  template <typename T, class CIn, class COut>
  static T ScanInclusive(const dax::cont::ArrayHandle<T, CIn, Tag>& input,
                         dax::cont::ArrayHandle<T, COut, Tag>& output) {
    return Scan(input, output, 0);
  }
  template <typename T, class CIn, class COut>
  static T ScanExclusive(const dax::cont::ArrayHandle<T, CIn, Tag>& input,
                         dax::cont::ArrayHandle<T, COut, Tag>& output) {
    return Scan(input, output, 1);
  }

  template <typename T, class Container>
  static void Sort(dax::cont::ArrayHandle<T, Container, Tag>& values) {
    SortImpl<T, char>(values.PrepareForInPlace().GetIteratorBegin(), nullptr,
                      values.GetNumberOfValues(), 0, 0);
  }

  template <typename T, typename U, class CKey, class CVal>
  static void SortByKey(dax::cont::ArrayHandle<T, CKey, Tag>& keys,
                        dax::cont::ArrayHandle<U, CVal, Tag>& values) {
    if (keys.GetNumberOfValues() != values.GetNumberOfValues())
      throw dax::cont::ErrorControlBadValue("SortByKey needs as many values as keys");
    SortImpl<T, U>(keys.PrepareForInPlace().GetIteratorBegin(),
                   values.PrepareForInPlace().GetIteratorBegin(), keys.GetNumberOfValues(),
                   (int)sizeof(U), 0);
  }

  /// The indices of the non-zero stencil entries (the one-argument form).
  template <typename T, class CStencil, class COut>
  static void StreamCompact(const dax::cont::ArrayHandle<T, CStencil, Tag>& stencil,
                            dax::cont::ArrayHandle<dax::Id, COut, Tag>& output) {
    Compact<dax::Id>(nullptr, stencil, output);
  }
  /// The input values whose stencil entry is non-zero, in order.
  template <typename T, typename U, class CIn, class CStencil, class COut>
  static void StreamCompact(const dax::cont::ArrayHandle<T, CIn, Tag>& input,
                            const dax::cont::ArrayHandle<U, CStencil, Tag>& stencil,
                            dax::cont::ArrayHandle<T, COut, Tag>& output) {
    if (input.GetNumberOfValues() != stencil.GetNumberOfValues())
      throw dax::cont::ErrorControlBadValue("StreamCompact needs a stencil entry per value");
    Compact<T>(input.PrepareForInput().GetIteratorBegin(), stencil, output);
  }

  template <typename T, class Container>
  static void Unique(dax::cont::ArrayHandle<T, Container, Tag>& values) {
    const dax::Id n = values.GetNumberOfValues();
    if (n == 0) return;
    T* d = values.PrepareForInPlace().GetIteratorBegin();
    const int type = dax::gb300::cont::internal::KeyType<T>();
    const size_t bytes = dax_gb300_compact_scratch_bytes(n, (int)sizeof(T));
    dax::gb300::cont::internal::DeviceBuffer scratch(bytes);
    int64_t kept = 0;
    dax::gb300::cont::internal::Check(
        dax_gb300_unique(d, n, type, scratch.Get(), bytes, &kept, nullptr));
    values.Shrink((dax::Id)kept);
  }

  static void Synchronize() { dax::gb300::cont::internal::Check(dax_gb300_synchronize(nullptr)); }

 private:
  template <typename T, class CIn, class CVal, class COut>
  static void Bounds(const dax::cont::ArrayHandle<T, CIn, Tag>& input,
                     const dax::cont::ArrayHandle<T, CVal, Tag>& values,
                     dax::cont::ArrayHandle<dax::Id, COut, Tag>& output, int upper) {
    const dax::Id n = input.GetNumberOfValues(), m = values.GetNumberOfValues();
    const T* in = input.PrepareForInput().GetIteratorBegin();
    const T* val = values.PrepareForInput().GetIteratorBegin();
    dax::Id* out = output.PrepareForOutput(m).GetIteratorBegin();
    dax::gb300::cont::internal::Check(dax_gb300_bounds(
        in, n, val, m, dax::gb300::cont::internal::KeyType<T>(), upper, out, nullptr));
    Synchronize();
  }

  template <class CIn, class COut>
  static void BoundsInPlace(const dax::cont::ArrayHandle<dax::Id, CIn, Tag>& input,
                            dax::cont::ArrayHandle<dax::Id, COut, Tag>& values_output,
                            int upper) {
    const dax::Id n = input.GetNumberOfValues(), m = values_output.GetNumberOfValues();
    const dax::Id* in = input.PrepareForInput().GetIteratorBegin();
    dax::Id* vo = values_output.PrepareForInPlace().GetIteratorBegin();
    dax::gb300::cont::internal::Check(dax_gb300_bounds(
        in, n, vo, m, dax::gb300::cont::internal::KeyType<dax::Id>(), upper, vo, nullptr));
    Synchronize();
  }

  template <typename T, class CIn, class COut>
  static T Scan(const dax::cont::ArrayHandle<T, CIn, Tag>& input,
                dax::cont::ArrayHandle<T, COut, Tag>& output, int exclusive) {
    const dax::Id n = input.GetNumberOfValues();
    T total = T();
    if (n == 0) {
      output.PrepareForOutput(0);
      return total;
    }
    const T* in = input.PrepareForInput().GetIteratorBegin();
    T* out = output.PrepareForOutput(n).GetIteratorBegin();
    const size_t bytes = dax_gb300_scan_scratch_bytes(n);
    dax::gb300::cont::internal::DeviceBuffer scratch(bytes);
    dax::gb300::cont::internal::Check(dax_gb300_scan(
        in, out, n, dax::gb300::cont::internal::KeyType<T>(), exclusive, scratch.Get(), bytes,
        &total, nullptr));
    return total;
  }

  template <typename T, typename U>
  static void SortImpl(T* keys, U* values, dax::Id n, int value_bytes, int descending) {
    if (n <= 1) return;
    const int type = dax::gb300::cont::internal::KeyType<T>();
    const size_t bytes = dax_gb300_sort_scratch_bytes(n, type, value_bytes);
    if (bytes == 0)
      throw dax::cont::ErrorControlBadValue("SortByKey values must be 4, 8, 12 or 16 bytes");
    dax::gb300::cont::internal::DeviceBuffer scratch(bytes);
    dax::gb300::cont::internal::Check(dax_gb300_sort_by_key(
        keys, values, n, type, value_bytes, descending, scratch.Get(), bytes, nullptr));
    Synchronize();
  }

  template <typename T, typename U, class CStencil, class COut>
  static void Compact(const T* input, const dax::cont::ArrayHandle<U, CStencil, Tag>& stencil,
                      dax::cont::ArrayHandle<T, COut, Tag>& output) {
    static_assert(sizeof(U) == 4, "the stencil is dax::Id or dax::Scalar");
    const dax::Id n = stencil.GetNumberOfValues();
    const U* st = stencil.PrepareForInput().GetIteratorBegin();
    T* out = output.PrepareForOutput(n).GetIteratorBegin();
    const size_t bytes = dax_gb300_compact_scratch_bytes(n, 0);
    dax::gb300::cont::internal::DeviceBuffer scratch(bytes);
    int64_t kept = 0;
    dax::gb300::cont::internal::Check(dax_gb300_stream_compact(
        input, input ? (int)sizeof(T) : 0, st, dax::gb300::cont::internal::KeyType<U>(), n, out,
        scratch.Get(), bytes, &kept, nullptr));
    output.Shrink((dax::Id)kept);
  }
};

}  // namespace cont
}  // namespace dax

namespace dax {
namespace gb300 {
namespace cont {

/// A uniform grid as the hot-path dispatchers take it: the fields of
/// dax::cont::UniformGrid (dax/cont/UniformGrid.h:114-252).
inline dax_gb300_uniform_grid MakeUniformGrid(const dax::Id3& dims,
                                              const dax::Vector3& origin = dax::Vector3(0.0f),
                                              const dax::Vector3& spacing = dax::Vector3(1.0f),
                                              const dax::Id3& extentMin = dax::Id3(0)) {
  dax_gb300_uniform_grid g;
  for (int a = 0; a < 3; ++a) {
    g.origin[a] = origin[a];
    g.spacing[a] = spacing[a];
    g.extent_min[a] = extentMin[a];
    g.extent_max[a] = extentMin[a] + dims[a] - 1;
  }
  return g;
}

typedef dax::cont::ArrayContainerControlTagBasic Basic;
typedef DeviceAdapterTagGB300 Tag;

/// DispatcherMapCell<MarchingCubesCount> then DispatcherGenerateInterpolatedCells
/// <MarchingCubesGenerate> with RemoveDuplicatePoints = removeDuplicates
/// (dax/cont/DispatcherGenerateInterpolatedCells.h:145-301): the triangle
/// connectivity (3 point ids per triangle) and the interpolated points.
inline void MarchingCubes(const dax_gb300_uniform_grid& grid,
                          const dax::cont::ArrayHandle<dax::Scalar, Basic, Tag>& field,
                          dax::Scalar isovalue, bool removeDuplicates,
                          dax::cont::ArrayHandle<dax::Id, Basic, Tag>& connectivity,
                          dax::cont::ArrayHandle<dax::Vector3, Basic, Tag>& points) {
  const float* f = field.PrepareForInput().GetIteratorBegin();
  const size_t bytes = dax_gb300_mc_scratch_bytes(&grid);
  if (bytes == 0) internal::Check(DAX_GB300_ERROR_BAD_VALUE);
  internal::DeviceBuffer scratch(bytes);
  internal::Check(dax_gb300_mc_count(&grid, f, isovalue, scratch.Get(), bytes, nullptr));
  int64_t T = 0, V = 0;
  internal::Check(dax_gb300_mc_totals(scratch.Get(), &T, &V, nullptr));
  if (!removeDuplicates) V = 3 * T;
  dax::Id* conn = connectivity.PrepareForOutput((dax::Id)(3 * T)).GetIteratorBegin();
  dax::Vector3* pts = points.PrepareForOutput((dax::Id)V).GetIteratorBegin();
  internal::Check(dax_gb300_mc_generate(&grid, f, isovalue, removeDuplicates ? 1 : 0,
                                        scratch.Get(), bytes, reinterpret_cast<float*>(pts), V,
                                        conn, T, nullptr, nullptr, nullptr, nullptr));
  internal::Check(dax_gb300_mc_totals(scratch.Get(), nullptr, nullptr, nullptr));
}

/// DispatcherMapCell<ThresholdCount> then DispatcherGenerateTopology
/// <ThresholdTopology> with RemoveDuplicatePoints and CompactPointField of the
/// field (dax/cont/DispatcherGenerateTopology.h:98-258): 8 point ids per
/// kept cell, the used points' coordinates and field values.
inline void Threshold(const dax_gb300_uniform_grid& grid,
                      const dax::cont::ArrayHandle<dax::Scalar, Basic, Tag>& field,
                      dax::Scalar thresholdMin, dax::Scalar thresholdMax,
                      dax::cont::ArrayHandle<dax::Id, Basic, Tag>& connectivity,
                      dax::cont::ArrayHandle<dax::Vector3, Basic, Tag>& points,
                      dax::cont::ArrayHandle<dax::Scalar, Basic, Tag>& pointField) {
  const float* f = field.PrepareForInput().GetIteratorBegin();
  const size_t bytes = dax_gb300_threshold_scratch_bytes(&grid);
  if (bytes == 0) internal::Check(DAX_GB300_ERROR_BAD_VALUE);
  internal::DeviceBuffer scratch(bytes);
  internal::Check(
      dax_gb300_threshold_count(&grid, f, thresholdMin, thresholdMax, scratch.Get(), bytes, nullptr));
  int64_t K = 0, U = 0;
  internal::Check(dax_gb300_threshold_totals(scratch.Get(), &K, &U, nullptr));
  dax::Id* conn = connectivity.PrepareForOutput((dax::Id)(8 * K)).GetIteratorBegin();
  dax::Vector3* pts = points.PrepareForOutput((dax::Id)U).GetIteratorBegin();
  float* pf = pointField.PrepareForOutput((dax::Id)U).GetIteratorBegin();
  internal::Check(dax_gb300_threshold_generate(&grid, f, thresholdMin, thresholdMax, scratch.Get(),
                                               bytes, conn, K, reinterpret_cast<float*>(pts), pf,
                                               U, nullptr));
  internal::Check(dax_gb300_threshold_totals(scratch.Get(), nullptr, nullptr, nullptr));
}

/// DispatcherMapCell<CellGradient> (dax/worklet/CellGradient.h:28-48): one
/// gradient per cell.
inline void CellGradient(const dax_gb300_uniform_grid& grid,
                         const dax::cont::ArrayHandle<dax::Scalar, Basic, Tag>& field,
                         dax::cont::ArrayHandle<dax::Vector3, Basic, Tag>& gradient) {
  dax::Id cells = 1;
  for (int a = 0; a < 3; ++a) {
    const dax::Id d = grid.extent_max[a] - grid.extent_min[a];
    cells *= d > 0 ? d : 0;
  }
  const float* f = field.PrepareForInput().GetIteratorBegin();
  dax::Vector3* g = gradient.PrepareForOutput(cells).GetIteratorBegin();
  internal::Check(dax_gb300_cell_gradient(&grid, f, reinterpret_cast<float*>(g), nullptr));
  internal::Check(dax_gb300_synchronize(nullptr));
}

}  // namespace cont
}  // namespace gb300
}  // namespace dax

#endif  // DAX_GB300_TAG_H
