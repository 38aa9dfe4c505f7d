"""Every transfer and fill of a system runs on the system's stream.

The stream of an imdgpu_sys is created non-blocking, so work issued on the
legacy default stream (plain cudaMemcpy / cudaMemset) is not ordered with
the kernels on it: a device-to-device copy or a fill there returns before it
has run.  A batch's replay after an overflow once restored its snapshot that
way, and the rebuild that followed on the system's stream read positions and
CG vectors half restored.  The sources that work on a system's stream use
stream-ordered helpers (scopy / sset) or the Async calls with the stream;
output.cu works on the legacy stream throughout and is not checked."""
import pathlib
import re

CSRC = pathlib.Path(__file__).resolve().parent.parent / "imd_gb300" / "csrc"
CHECKED = ["system.cu", "forces.cu", "mixed.cu", "batch.cu", "learn.cu"]


def _code(text: str) -> str:
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.sub(r"//[^\n]*", "", text)


def test_no_legacy_stream_transfers():
    found = []
    for name in CHECKED:
        code = _code((CSRC / name).read_text())
        for m in re.finditer(r"\bcuda(Memcpy|Memset)(2D|3D|ToSymbol|FromSymbol)?\s*\(", code):
            line = code[:m.start()].count("\n") + 1
            found.append("%s:%d %s" % (name, line, m.group(0)))
    assert not found, found


def test_async_calls_name_a_stream():
    """cudaMemcpyAsync / cudaMemsetAsync without a stream argument, or with
    stream 0, would be on the legacy stream as well."""
    found = []
    for name in CHECKED:
        code = _code((CSRC / name).read_text())
        for m in re.finditer(r"\bcuda(MemcpyAsync|MemsetAsync)\s*\(([^;]*)\)\s*;", code):
            last = m.group(2).rsplit(",", 1)[-1].strip()
            if last in ("0", "nullptr", "NULL", "cudaStreamLegacy"):
                found.append("%s: %s" % (name, m.group(0)[:80]))
    assert not found, found
