"""The binding INTEGRATION.md shows a maintainer adding to the reference's
graph.cpp (gpuConstructAndCutoff, in place of constructDistNodeGraph +
cutoffGraph, graph.cpp:3479,3544) compiles against the reference's own
sources and links against libswapgb.so. The code block is taken from
INTEGRATION.md itself, so the document cannot drift from what compiles.
On a machine without a GPU the linked program runs up to the library's
device check and exits with its error (nothing falls back to the CPU)."""
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
ORACLE = ROOT / "oracle"
REF_FILE = ORACLE / "_ref" / "REF"
PKG = ROOT / "swap-assembler_gb300"

DRIVER = r'''// generated by tests/test_integration_binding.py: the reference's graph.cpp
// (main renamed) plus the binding of INTEGRATION.md, then the reference's main
// sequence with the binding in place of construction + cutoff.
#define main swap_reference_main
#include "graph.cpp"
#undef main
#include <cstring>
#include <vector>

%s

int main(int argc, char *argv[]) {
    MPIEnviroment MPIcontrol;
    MPIcontrol.init(argc, argv);
    parameter parameters;
    parameters.getParameters(argc, argv, &MPIcontrol);
    distNodeGraph *nodeGraph = new distNodeGraph(&parameters, &MPIcontrol);
    if (getenv("SWG_HOST_FRAMING")) gpuConstructAndCutoffHostFraming(nodeGraph, &parameters);
    else gpuConstructAndCutoff(nodeGraph, &parameters);
    nodeGraph->buildKmoleculeGraph(&MPIcontrol, &parameters);
    nodeGraph->graphStatistics(&parameters, &MPIcontrol);
    strcpy(parameters.kmerGraph, parameters.outputPath);
    strcat(parameters.kmerGraph, "/nodes.txt");
    nodeGraph->printLocalNodeGraph(&parameters, &MPIcontrol);
    MPIcontrol.finalize();
    return 0;
}
'''


def binding_blocks() -> str:
    """Both bindings INTEGRATION.md shows: device framing from the file (the
    one main calls) and host framing."""
    text = (ROOT / "INTEGRATION.md").read_text()
    blocks = re.findall(r"```cpp\n(.*?)```", text, flags=re.S)
    got = [b for b in blocks if "static void gpuConstructAndCutoff" in b]
    assert len(got) == 2, "expected the device- and host-framing bindings"
    return "\n".join(got)


@pytest.fixture(scope="module")
def ref_dir() -> Path:
    if not REF_FILE.exists():
        pytest.skip("the reference was not compiled here (oracle/_ref)")
    d = Path(REF_FILE.read_text().strip())
    if not (d / "graph.cpp").exists():
        pytest.skip("reference sources not present")
    return d


def test_binding_compiles_and_links(ref_dir, tmp_path):
    src = tmp_path / "binding.cpp"
    src.write_text(DRIVER % binding_blocks())
    objs = [ORACLE / "_ref" / n for n in ("kmerGraph.o", "sequence.o", "mympi.o", "mpi_shim.o")]
    for o in objs:
        assert o.exists(), o
    exe = tmp_path / "swap_gpu"
    cmd = ["g++", "-O1", "-w", "-Wno-deprecated", "-I" + str(ORACLE / "mpishim"), "-I" + str(ref_dir),
           "-I" + str(ROOT / "include"), str(src), *map(str, objs), "-L" + str(PKG), "-lswapgb",
           "-Wl,-rpath," + str(PKG), "-lpthread", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # run it: without a GPU the build returns its no-device error and the
    # binding exits 1 with that message
    fa = tmp_path / "r.fa"
    fa.write_bytes(b">r1\n" + b"ACGTTGCAAGGCTTACCGATCGATCGGATCCATG" * 3 + b"\n")
    out = tmp_path / "out"
    p = subprocess.run([str(exe), "-k", "21", "-c", "1", "-i", str(fa), "-o", str(out)],
                       capture_output=True, text=True, timeout=120)
    import torch
    if not torch.cuda.is_available():
        assert p.returncode == 1 and "Error:" in p.stdout
