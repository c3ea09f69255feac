"""The C ABI library loads and exports every entry point the header declares.

No compute call is made here (no GPU needed); the symbol set and the buffer
and value counts are checked against ``include/sand_dem_gb300.h`` and the
host-side buffer order.
"""

import ctypes as ct
import re
from pathlib import Path

import pytest

from sand_atlas_dem_gb300 import native
from sand_atlas_dem_gb300.engine import BUFFER_ORDER, EXTENSION_ORDER, TUNING_KEYS
from sand_atlas_dem_gb300.model import CONFIG_ORDER, RESOURCE_ORDER

HEADER = Path(__file__).resolve().parent.parent / "include" / "sand_dem_gb300.h"


def declared():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(sdg_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def library():
    if not native.LIBRARY.exists():
        native.build()
    return ct.CDLL(str(native.LIBRARY))


def test_header_and_exports_agree(library):
    names = declared()
    assert set(names) == set(native.EXPORTS)
    for name in names:
        assert hasattr(library, name), name


def test_buffer_and_value_counts(library):
    text = HEADER.read_text()
    buffers = int(re.search(r"#define SDG_BUFFER_COUNT (\d+)", text)[1])
    values = int(re.search(r"#define SDG_VALUE_COUNT (\d+)", text)[1])
    library.sdg_buffer_count.restype = ct.c_int
    library.sdg_value_count.restype = ct.c_int
    assert library.sdg_buffer_count() == buffers == len(BUFFER_ORDER) == len(RESOURCE_ORDER) + len(EXTENSION_ORDER)
    assert library.sdg_value_count() == values == len(CONFIG_ORDER) + 5 + len(TUNING_KEYS) + 3
    assert len(RESOURCE_ORDER) == 77


def test_argument_errors_are_reported_without_a_device(library):
    lib = native.load()
    rc = lib.sdg_dispatch(b"beginStep", 1, None, None, None, 0, None)
    assert rc == 1
    assert b"buffers" in lib.sdg_last_error()


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    monkeypatch.setattr(native, "_LIB", None)
    monkeypatch.setattr(native, "LIBRARY", tmp_path / "absent.so")
    with pytest.raises(RuntimeError, match="not built"):
        native.load()


def test_host_sizes_match_device_constants():
    """Buffer sizes the host computes use the device layout's constants."""
    from sand_atlas_dem_gb300 import engine

    text = (native.CSRC / "dem_device.cuh").read_text()
    cells = int(re.search(r"constexpr uint32_t WALK_CELLS = (\d+);", text)[1])
    grid = int(re.search(r"constexpr uint32_t GRID = (\d+);", text)[1])
    assert engine.WALK_BUCKETS == cells**3
    assert engine.DISTANCE_GRID == grid
