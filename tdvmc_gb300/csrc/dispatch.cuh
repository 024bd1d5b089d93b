// Kernel dispatch tables; the template instantiations live in the
// inst_*.cu translation units so the library builds in parallel.
#pragma once

#include "common.cuh"
#include "k_sample.cuh"

namespace tdvmc {

template <typename T>
using SampleFn = void (*)(SysConst, const Q4<T>*, const T*, const T*, const T*, const int*, T*, int64_t, int64_t,
                          const int32_t*, int, T, uint2, const uint32_t*, int*);
template <typename T>
using ElocFn = void (*)(SysConst, const DynState*, const Q4<T>*, const T*, const T*, const int*, const T*,
                        const double*, const double*, const T*, int64_t, T*, T*, T*, T*, T*, T*);
template <typename T>
using RevFn = void (*)(SysConst, const T*, const T*, const int*, const T*, const double*, const T*, const T*, int64_t,
                       T*);

// register slots per lane available for `lanes` lanes per walker
int sample_slots_for(int n, int lanes);

SampleFn<float> pick_sample_f32(int lanes, int slots);
// FP32, uniform knots: packed f32x2 pair arithmetic (null where not instantiated)
SampleFn<float> pick_sample_f32_packed(int lanes, int slots);
// the same with the lane's coordinates in shared memory (null where not instantiated)
SampleFn<float> pick_sample_f32_packed_shared(int lanes, int slots);
SampleFn<double> pick_sample_f64(int lanes, int slots);
ElocFn<float> pick_eloc_f32(int lanes, bool adj, int hist);
ElocFn<double> pick_eloc_f64(int lanes, bool adj, int hist);
RevFn<float> pick_eloc_rev_f32(int lanes, int hist);
RevFn<double> pick_eloc_rev_f64(int lanes, int hist);

// NUBosonsBulkPB (mirrored distances): 32 lanes, histogram mode 0, the scalar
// sampler; null for any other tile
template <typename T> SampleFn<T> pick_sample_pb(int lanes, int slots);
SampleFn<float> pick_sample_f32_packed_pb(int lanes, int slots);  // FP32, uniform knots
template <typename T> ElocFn<T> pick_eloc_pb(int lanes, bool adj, int hist);
template <typename T> RevFn<T> pick_eloc_rev_pb(int lanes, int hist);
template <> SampleFn<float> pick_sample_pb<float>(int lanes, int slots);
template <> SampleFn<double> pick_sample_pb<double>(int lanes, int slots);
template <> ElocFn<float> pick_eloc_pb<float>(int lanes, bool adj, int hist);
template <> ElocFn<double> pick_eloc_pb<double>(int lanes, bool adj, int hist);
template <> RevFn<float> pick_eloc_rev_pb<float>(int lanes, int hist);
template <> RevFn<double> pick_eloc_rev_pb<double>(int lanes, int hist);

template <typename T> SampleFn<T> pick_sample(int lanes, int slots);
template <> inline SampleFn<float> pick_sample<float>(int g, int s) { return pick_sample_f32(g, s); }
template <> inline SampleFn<double> pick_sample<double>(int g, int s) { return pick_sample_f64(g, s); }
template <typename T> ElocFn<T> pick_eloc(int lanes, bool adj, int hist);
template <> inline ElocFn<float> pick_eloc<float>(int g, bool a, int h) { return pick_eloc_f32(g, a, h); }
template <> inline ElocFn<double> pick_eloc<double>(int g, bool a, int h) { return pick_eloc_f64(g, a, h); }
template <typename T> RevFn<T> pick_eloc_rev(int lanes, int hist);
template <> inline RevFn<float> pick_eloc_rev<float>(int g, int h) { return pick_eloc_rev_f32(g, h); }
template <> inline RevFn<double> pick_eloc_rev<double>(int g, int h) { return pick_eloc_rev_f64(g, h); }

}  // namespace tdvmc
