#include "dispatch.cuh"
#define TDVMC_T float
#define TDVMC_FN pick_sample_f32
#include "inst_sample.inc"
namespace tdvmc {
int sample_slots_for(int n, int G) {
	static const int l32[] = {1, 2, 4, 8, 11, 16, 32};
	static const int l16[] = {1, 2, 4, 8, 16, 22};
	static const int l8[] = {1, 2, 4};
	const int need = (n + G - 1) / G;
	const int* l = G == 32 ? l32 : (G == 16 ? l16 : l8);
	const int m = G == 32 ? 7 : (G == 16 ? 6 : 3);
	if (G != 32 && G != 16 && G != 8) return -1;
	for (int i = 0; i < m; i++)
		if (l[i] >= need) return l[i];
	return -1;
}

SampleFn<float> pick_sample_f32_packed_shared(int G, int slots) {
	if (G == 32) {
		switch (slots) {
		case 8: return k_sample_f2<32, 8, true>;
		case 11: return k_sample_f2<32, 11, true>;
		case 16: return k_sample_f2<32, 16, true>;
		case 32: return k_sample_f2<32, 32, true>;
		}
	} else if (G == 16) {
		switch (slots) {
		case 16: return k_sample_f2<16, 16, true>;
		case 22: return k_sample_f2<16, 22, true>;
		}
	}
	return nullptr;
}

SampleFn<float> pick_sample_f32_packed(int G, int slots) {
	if (G == 32) {
		switch (slots) {
		case 1: return k_sample_f2<32, 1>;
		case 2: return k_sample_f2<32, 2>;
		case 4: return k_sample_f2<32, 4>;
		case 8: return k_sample_f2<32, 8>;
		case 11: return k_sample_f2<32, 11>;
		case 16: return k_sample_f2<32, 16>;
		case 32: return k_sample_f2<32, 32, true>;
		}
	} else if (G == 16) {
		switch (slots) {
		case 1: return k_sample_f2<16, 1>;
		case 2: return k_sample_f2<16, 2>;
		case 4: return k_sample_f2<16, 4>;
		case 8: return k_sample_f2<16, 8>;
		case 16: return k_sample_f2<16, 16>;
		case 22: return k_sample_f2<16, 22>;
		}
	} else if (G == 8) {
		switch (slots) {
		case 1: return k_sample_f2<8, 1>;
		case 2: return k_sample_f2<8, 2>;
		case 4: return k_sample_f2<8, 4>;
		}
	}
	return nullptr;
}
}  // namespace tdvmc
