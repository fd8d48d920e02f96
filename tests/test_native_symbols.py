"""The C-ABI library loads and exports every entry point include/*.h declares (CPU only)."""
import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for header in glob.glob(os.path.join(ROOT, "include", "**", "*.h"), recursive=True):
        text = open(header).read()
        names += re.findall(r"FASTNOISE_API\s+[\w\s\*]+?\b(fn\w+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_reference_entry_points():
    names = declared_symbols()
    # every generation and metadata entry point of the reference FastNoise_C.h
    for ref in ["fnNewFromEncodedNodeTree", "fnDeleteNodeRef", "fnGetActiveFeatureSet", "fnGetMetadataID",
                "fnGenUniformGrid2D", "fnGenUniformGrid3D", "fnGenUniformGrid4D", "fnGenPositionArray2D",
                "fnGenPositionArray3D", "fnGenPositionArray4D", "fnGenTileable2D", "fnGenSingle2D", "fnGenSingle3D",
                "fnGenSingle4D", "fnGetMetadataCount", "fnGetMetadataName", "fnNewFromMetadata",
                "fnGetMetadataVariableCount", "fnGetMetadataVariableName", "fnGetMetadataVariableType",
                "fnGetMetadataVariableDimensionIdx", "fnGetMetadataEnumCount", "fnGetMetadataEnumName",
                "fnSetVariableFloat", "fnSetVariableIntEnum", "fnGetMetadataNodeLookupCount",
                "fnGetMetadataNodeLookupName", "fnGetMetadataNodeLookupDimensionIdx", "fnSetNodeLookup",
                "fnGetMetadataHybridCount", "fnGetMetadataHybridName", "fnGetMetadataHybridDimensionIdx",
                "fnSetHybridNodeLookup", "fnSetHybridFloat", "fnGetMetadataDescription", "fnGetMetadataGroupCount",
                "fnGetMetadataGroupName", "fnGetMetadataVariableDescription", "fnGetMetadataVariableDefaultFloat",
                "fnGetMetadataVariableDefaultIntEnum", "fnGetMetadataVariableMinFloat",
                "fnGetMetadataVariableMaxFloat", "fnGetMetadataNodeLookupDescription",
                "fnGetMetadataHybridDescription", "fnGetMetadataHybridDefault"]:
        assert ref in names, ref


def test_library_exports_every_declared_symbol(native):
    lib = ctypes.CDLL(native.library_path())
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
