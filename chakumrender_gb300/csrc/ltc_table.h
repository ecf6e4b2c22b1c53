// ltc_table.h — the GGX LTC fit table (FP32 device form) and its loader.
#pragma once
#include <vector>

#include "shading_device.cuh"

namespace ckr {

// Loads data/ltc_ggx.bin (path, or the copy next to libckr.so when path is
// NULL) into 4096 FP32 entries.  Returns CKR_OK or CKR_ERR_IO / CKR_ERR_PARSE.
int load_ltc_table(const char *path, std::vector<LtcEntry> &out);

// Device copy for the current device (loaded on first use); nullptr on failure.
const LtcEntry *device_ltc_table(int *status);

}  // namespace ckr
