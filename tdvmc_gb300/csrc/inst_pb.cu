// Instantiations for NUBosonsBulkPB (mirrored pair distances): the scalar
// sampler and the evaluation kernels with 32-lane groups and histogram mode 0,
// both arithmetic types.
#include "dispatch.cuh"
#include "k_eloc.cuh"

namespace tdvmc {

template <typename T>
static SampleFn<T> pick_sample_pb_t(int lanes, int slots) {
	if (lanes != 32) return nullptr;
	switch (slots) {
	case 1: return k_sample<T, 32, 1, true>;
	case 2: return k_sample<T, 32, 2, true>;
	case 4: return k_sample<T, 32, 4, true>;
	case 8: return k_sample<T, 32, 8, true>;
	case 11: return k_sample<T, 32, 11, true>;
	case 16: return k_sample<T, 32, 16, true>;
	case 32: return k_sample<T, 32, 32, true>;
	}
	return nullptr;
}
template <> SampleFn<float> pick_sample_pb<float>(int lanes, int slots) { return pick_sample_pb_t<float>(lanes, slots); }
SampleFn<float> pick_sample_f32_packed_pb(int lanes, int slots) {
	if (lanes != 32) return nullptr;
	switch (slots) {
	case 1: return k_sample_f2<32, 1, false, true>;
	case 2: return k_sample_f2<32, 2, false, true>;
	case 4: return k_sample_f2<32, 4, false, true>;
	case 8: return k_sample_f2<32, 8, false, true>;
	case 11: return k_sample_f2<32, 11, false, true>;
	case 16: return k_sample_f2<32, 16, false, true>;
	case 32: return k_sample_f2<32, 32, true, true>;
	}
	return nullptr;
}
template <> SampleFn<double> pick_sample_pb<double>(int lanes, int slots) { return pick_sample_pb_t<double>(lanes, slots); }

template <> ElocFn<float> pick_eloc_pb<float>(int lanes, bool adj, int hist) {
	if (lanes != 32 || hist != 0) return nullptr;
	return adj ? k_eloc<float, 32, true, 0, true> : k_eloc<float, 32, false, 0, true>;
}
template <> ElocFn<double> pick_eloc_pb<double>(int lanes, bool adj, int hist) {
	if (lanes != 32 || hist != 0) return nullptr;
	return adj ? k_eloc<double, 32, true, 0, true> : k_eloc<double, 32, false, 0, true>;
}
template <> RevFn<float> pick_eloc_rev_pb<float>(int lanes, int hist) {
	return (lanes == 32 && hist == 0) ? k_eloc_rev<float, 32, 0, true> : nullptr;
}
template <> RevFn<double> pick_eloc_rev_pb<double>(int lanes, int hist) {
	return (lanes == 32 && hist == 0) ? k_eloc_rev<double, 32, 0, true> : nullptr;
}

}  // namespace tdvmc
