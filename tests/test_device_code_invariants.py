"""Source-level invariants of the CUDA kernels, checked without a GPU.

* Every mbarrier wait is bounded: each ``mbarrier.try_wait`` sits in a
  helper whose poll loop has an iteration limit, and the helper reports
  whether the wait gave up (the kernels turn that into the status word the
  host reads as SUBBY_ERR_TIMEOUT).
* Tensor memory is returned as allocated: in each source file the column
  counts given to ``tcgen05.dealloc`` are the ones given to
  ``tcgen05.alloc`` (a power of two, 32..512)."""
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SOURCES = sorted(glob.glob(os.path.join(ROOT, "subby_gb300", "csrc", "*.cu")) +
                 glob.glob(os.path.join(ROOT, "subby_gb300", "csrc", "*.cuh")))


def _read(path):
    with open(path) as f:
        return f.read()


def test_sources_found():
    names = {os.path.basename(p) for p in SOURCES}
    assert {"k_big.cu", "k_tree4.cu", "walk.cuh", "k_acctc.cu"} <= names


def test_every_mbarrier_wait_is_bounded():
    helper = re.compile(r"bool\s+(\w+)\s*\(uint32_t mb, uint32_t phase[^)]*\)\s*\{")
    sites = 0
    for path in SOURCES:
        src = _read(path)
        for m in re.finditer(r"mbarrier\.try_wait", src):
            sites += 1
            # the enclosing helper: the last helper signature before the site
            heads = [h for h in helper.finditer(src) if h.end() <= m.start()]
            assert heads, f"{os.path.basename(path)}: try_wait outside a wait helper"
            body = src[heads[-1].end():m.start()]
            assert re.search(r"for \(int it = 0; it < \w+; \+\+it\)", body), \
                f"{os.path.basename(path)}:{heads[-1].group(1)} has no poll limit"
            tail = src[m.end():m.end() + 400]
            assert "if (done) return true;" in tail and "return false;" in tail, \
                f"{os.path.basename(path)}:{heads[-1].group(1)} does not report a wait that gave up"
    assert sites >= 2


def _column_counts(src, op):
    """Column count of each ``tcgen05.<op>``: its first numeric "r"(N)
    operand, within the asm statement (a short window after the opcode)."""
    out = []
    for m in re.finditer(r"tcgen05\." + op + r"\.cta_group::1", src):
        n = re.search(r'"r"\((\d+)\)', src[m.end():m.end() + 300])
        out.append(int(n.group(1)) if n else None)
    return out


def test_tensor_memory_deallocated_as_allocated():
    files = 0
    for path in SOURCES:
        src = _read(path)
        name = os.path.basename(path)
        a, d = _column_counts(src, "alloc"), _column_counts(src, "dealloc")
        if not a:
            assert not d, name
            continue
        files += 1
        assert None not in a and None not in d, f"{name}: a column count is not a literal"
        assert len(d) >= len(a), name
        assert set(a) == set(d), f"{name}: allocates {sorted(set(a))} columns, deallocates {sorted(set(d))}"
        for cols in a:
            assert 32 <= cols <= 512 and cols & (cols - 1) == 0, f"{name}: {cols} columns"
    assert files >= 4
