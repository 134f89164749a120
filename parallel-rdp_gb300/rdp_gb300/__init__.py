"""Python host API of the GB300-native N64 RDP path.

`CommandProcessor` mirrors the reference's RDP::CommandProcessor
(parallel-rdp/rdp_device.hpp:111-197) method for method, over the C ABI of
librdp_cuda.so (include/rdp_cuda.h).  There is no CPU fallback: importing this
package fails loudly when the native library has not been built.
"""
from .native import (  # noqa: F401
    Batch,
    CommandProcessor,
    RdpError,
    RdpTimeout,
    ScanoutOptions,
    VIRegister,
    SHADE_ORDERS,
    SHADE_VARIANTS,
    device_is_supported,
    get_shade_order,
    get_shade_variant,
    mlp_forward,
    mlp_gradients,
    MLP_PARAMS,
    set_shade_order,
    set_shade_variant,
    library_path,
)
from .cmdgen import GenParams, generate_stream, CONFIG_PLAIN, CONFIG_TEXTURED, CONFIG_MIXED  # noqa: F401
