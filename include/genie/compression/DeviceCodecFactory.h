// genie/compression/DeviceCodecFactory.h -- the codec ids of the reference
// (src/genie/compression/DeviceCodecFactory.h:38-53), as the legacy
// configuration names them.  Values equal enum genie_codec of <genie_gb300.h>.
#ifndef GENIE_COMPRESSION_DEVICECODECFACTORY_H_
#define GENIE_COMPRESSION_DEVICECODECFACTORY_H_

namespace genie {
namespace compression {

enum COMPRESSION_TYPE {
    NO_COMPRESSION = 0, COPY, DELTA, BP32, VARINT, COMP_BP32_COPY, COMP_BP32_VARINT, SERIAL_COPY_COPY,
    SERIAL_DELTA_COPY, SERIAL_DELTA_DELTA, SERIAL_DELTA_VARINT, SERIAL_DELTA_BP32, SERIAL_DELTA_COMP_BP32_COPY,
    SERIAL_DELTA_COMP_BP32_VARINT
};

// A table built from a configuration with no codec set is uncompressed.
const COMPRESSION_TYPE DEFAULT_COMPRESSION_TYPE = NO_COMPRESSION;

}  // namespace compression
}  // namespace genie

#endif
