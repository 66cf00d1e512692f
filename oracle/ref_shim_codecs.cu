// ref_shim_codecs.cu -- TEST INFRASTRUCTURE ONLY.
//
// Compiles the reference's own host codec encoders/decoders from the read-only
// reference tree (src/genie/compression/*.cu, included by path from the
// include directory given on the command line) into oracle/_ref/, and exposes
// them through a plain C ABI so that tests/golden/make_golden.py can pin the
// oracle's codec formats byte for byte.  Nothing here ships; the built library
// stays out of version control.
#include <cstdint>
#include <cstdarg>
#include <cstring>

#include "genie/utility/scan.cu"
#include "genie/compression/DeviceCodecs.cu"
#include "genie/compression/DeviceBitPackingHelpers.cu"
#include "genie/compression/DeviceBitPackingCodec.cu"
#include "genie/compression/DeviceVarintCodec.cu"
#include "genie/compression/DeviceCompositeCodec.cu"
#include "genie/compression/DeviceSerialCodec.cu"

// The codec sources reference the logger only on error paths.
const char *const genie::utility::Logger::LEVEL_NAMES[] = {"NONE", "ALERT", "INFO", "VERBOSE", "DEBUG"};
int genie::utility::Logger::log(int, const char *, ...) { return 0; }

using namespace genie::compression;

template <class C>
static int64_t enc(const uint32_t *in, int64_t n, uint32_t *out, int64_t cap) {
    C codec;
    size_t nvalue = (size_t)cap;
    codec.encodeArray(const_cast<uint32_t *>(in), (size_t)n, out, nvalue);
    return (int64_t)nvalue;
}

template <class C>
static int64_t dec(const uint32_t *in, int64_t nw, uint32_t *out, int64_t cap) {
    C codec;
    size_t nvalue = (size_t)cap;
    codec.decodeArray(in, (size_t)nw, out, nvalue);
    return (int64_t)nvalue;
}

typedef DeviceCompositeCodec<DeviceBitPackingCodec, DeviceCopyCodec> CBC;
typedef DeviceCompositeCodec<DeviceBitPackingCodec, DeviceVarintCodec> CBV;

// codec ids follow the reference COMPRESSION_TYPE enum (DeviceCodecFactory.h:38-53)
extern "C" int64_t ref_encode(int codec, const uint32_t *in, int64_t n, uint32_t *out, int64_t cap) {
    switch (codec) {
    case 1: return enc<DeviceCopyCodec>(in, n, out, cap);
    case 2: return enc<DeviceDeltaCodec>(in, n, out, cap);
    case 3: return enc<DeviceBitPackingCodec>(in, n, out, cap);
    case 4: return enc<DeviceVarintCodec>(in, n, out, cap);
    case 5: return enc<CBC>(in, n, out, cap);
    case 6: return enc<CBV>(in, n, out, cap);
    case 7: return enc<DeviceSerialCodec<DeviceCopyCodec, DeviceCopyCodec>>(in, n, out, cap);
    case 8: return enc<DeviceSerialCodec<DeviceDeltaCodec, DeviceCopyCodec>>(in, n, out, cap);
    case 9: return enc<DeviceSerialCodec<DeviceDeltaCodec, DeviceDeltaCodec>>(in, n, out, cap);
    case 10: return enc<DeviceSerialCodec<DeviceDeltaCodec, DeviceVarintCodec>>(in, n, out, cap);
    case 11: return enc<DeviceSerialCodec<DeviceDeltaCodec, DeviceBitPackingCodec>>(in, n, out, cap);
    case 12: return enc<DeviceSerialCodec<DeviceDeltaCodec, CBC>>(in, n, out, cap);
    case 13: return enc<DeviceSerialCodec<DeviceDeltaCodec, CBV>>(in, n, out, cap);
    }
    return -1;
}

extern "C" int64_t ref_decode(int codec, const uint32_t *in, int64_t nw, uint32_t *out, int64_t cap) {
    switch (codec) {
    case 1: return dec<DeviceCopyCodec>(in, nw, out, cap);
    case 2: return dec<DeviceDeltaCodec>(in, nw, out, cap);
    case 3: return dec<DeviceBitPackingCodec>(in, nw, out, cap);
    case 4: return dec<DeviceVarintCodec>(in, nw, out, cap);
    case 5: return dec<CBC>(in, nw, out, cap);
    case 6: return dec<CBV>(in, nw, out, cap);
    case 7: return dec<DeviceSerialCodec<DeviceCopyCodec, DeviceCopyCodec>>(in, nw, out, cap);
    case 8: return dec<DeviceSerialCodec<DeviceDeltaCodec, DeviceCopyCodec>>(in, nw, out, cap);
    case 9: return dec<DeviceSerialCodec<DeviceDeltaCodec, DeviceDeltaCodec>>(in, nw, out, cap);
    case 10: return dec<DeviceSerialCodec<DeviceDeltaCodec, DeviceVarintCodec>>(in, nw, out, cap);
    case 11: return dec<DeviceSerialCodec<DeviceDeltaCodec, DeviceBitPackingCodec>>(in, nw, out, cap);
    case 12: return dec<DeviceSerialCodec<DeviceDeltaCodec, CBC>>(in, nw, out, cap);
    case 13: return dec<DeviceSerialCodec<DeviceDeltaCodec, CBV>>(in, nw, out, cap);
    }
    return -1;
}
