"""GB300-native Sentinel-1 Level-0 -> SLC hot path (sm_103a CUDA behind a C ABI).

`S1Decoder` mirrors the reference's S1_Decoder; `build()` compiles the
in-tree CUDA library; `synth` makes seeded synthetic Level-0 streams.
"""
from .build import build  # noqa: F401
from .decoder import (AZIMUTH_COMPRESSED, CF32, CF64, EXPORTS, LEVELS, RANGE_COMPRESSED,  # noqa: F401
                      RANGE_DOPPLER, RAW, S1Decoder, S1GError, batch_outputs, launch_count,
                      annotation_times, load_library, process_swath_batch, read_annotation, read_index,
                      sidecar_paths, write_tiff)
