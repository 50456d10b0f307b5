"""Bit-exact parity against the reference's own GPU kernels.

apsepKernelSPT (src/apsep.cuh:2634, int32 keys, <BLOCK_SIZE = 128, IPT = 4>,
both comparators) is built from the reference sources into device code only
(oracle/_ref/apsep_ref_spt.ptx, by oracle/build_ref.py) and launched here
through the CUDA driver API the way runSPT launches it
(src/apsep.cuh:3052-3067): one cooperative launch of occupancy x SM-count
blocks of 128 threads over the five scratch arrays of allocSPTScratch
(src/apsep.cuh:3014-3040).  The reference's generic multi-kernel path, WSTL
(src/apsep.cuh:2296-2500, strict comparator), comes from the same module for
int32 and float32 keys and runs as runWSTL runs it (src/apsep.cuh:2548-2596):
the reference's own GPU oracle for float keys.  The engine must give the same
answers on the same inputs; the reference kernels are the checkers, never the
thing measured.
Skipped when the PTX was not built (no reference checkout where the
repository was built)."""
import ctypes
import os

import numpy as np
import pytest
import torch

from apsep_gb300 import Plan
from oracle import build_ref

pytestmark = pytest.mark.gpu

_vp, _u32 = ctypes.c_void_p, ctypes.c_uint


class ReferenceKernels:
    """The reference's kernels from oracle/_ref/apsep_ref_spt.ptx, launched
    as its host functions launch them."""

    def __init__(self):
        if not os.path.isfile(build_ref.SPT_PTX):
            pytest.skip("the reference kernel's PTX was not built (no reference checkout)")
        torch.zeros(1, device="cuda")  # the primary context, current on this thread
        cu = ctypes.CDLL("libcuda.so.1")
        for name in ("cuModuleGetFunctionCount", "cuModuleEnumerateFunctions", "cuFuncGetName"):
            if not hasattr(cu, name):
                pytest.skip("driver without %s" % name)
        cu.cuModuleLoadData.argtypes = [ctypes.POINTER(_vp), ctypes.c_char_p]
        cu.cuModuleUnload.argtypes = [_vp]
        cu.cuModuleGetFunctionCount.argtypes = [ctypes.POINTER(_u32), _vp]
        cu.cuModuleEnumerateFunctions.argtypes = [ctypes.POINTER(_vp), _u32, _vp]
        cu.cuFuncGetName.argtypes = [ctypes.POINTER(ctypes.c_char_p), _vp]
        cu.cuOccupancyMaxActiveBlocksPerMultiprocessor.argtypes = [ctypes.POINTER(ctypes.c_int), _vp,
                                                                   ctypes.c_int, ctypes.c_size_t]
        cu.cuLaunchCooperativeKernel.argtypes = [_vp, _u32, _u32, _u32, _u32, _u32, _u32, _u32, _vp,
                                                 ctypes.POINTER(_vp)]
        self.cu = cu
        with open(build_ref.SPT_PTX, "rb") as f:
            ptx = f.read() + b"\0"
        self.mod = _vp()
        self._check(cu.cuModuleLoadData(ctypes.byref(self.mod), ptx), "cuModuleLoadData")
        count = _u32()
        self._check(cu.cuModuleGetFunctionCount(ctypes.byref(count), self.mod), "cuModuleGetFunctionCount")
        funcs = (_vp * count.value)()
        self._check(cu.cuModuleEnumerateFunctions(funcs, count, self.mod), "cuModuleEnumerateFunctions")
        self.names = {}
        for f in funcs:
            name = ctypes.c_char_p()
            self._check(cu.cuFuncGetName(ctypes.byref(name), f), "cuFuncGetName")
            self.names[name.value] = _vp(f)
        self.fn = {incl: self.function(b"apsepKernelSPTIiLi128ELi4E" + tag)
                   for incl, tag in ((False, b"Lb0E"), (True, b"Lb1E"))}
        cu.cuLaunchKernel.argtypes = [_vp, _u32, _u32, _u32, _u32, _u32, _u32, _u32, _vp, ctypes.POINTER(_vp), _vp]
        self.sms = torch.cuda.get_device_properties(0).multi_processor_count

    def function(self, part: bytes):
        """The module's one function whose mangled name contains `part`."""
        hits = [f for nm, f in self.names.items() if part in nm]
        assert len(hits) == 1, "kernel %r not found once in the module" % part
        return hits[0]

    def _launch(self, f, grid, block, vals, cooperative=False):
        args = (_vp * len(vals))(*[ctypes.cast(ctypes.byref(v), _vp) for v in vals])
        stream = _vp(torch.cuda.current_stream().cuda_stream)
        if cooperative:
            rc = self.cu.cuLaunchCooperativeKernel(f, grid, 1, 1, block, 1, 1, 0, stream, args)
        else:
            rc = self.cu.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, stream, args, None)
        self._check(rc, "kernel launch")

    def run_wstl(self, x: torch.Tensor) -> torch.Tensor:
        """runWSTL (src/apsep.cuh:2548-2596): pass 1 per block, the block-min
        tree bottom-up level by level, pass 3 for the unresolved keys."""
        t = {torch.int32: b"i", torch.float32: b"f"}[x.dtype]
        n = x.numel()
        B, W = 512, 16
        nb = (n + B - 1) // B
        M = 1
        while M < nb:
            M <<= 1
        dev = x.device
        leaves = torch.empty(nb * B, dtype=x.dtype, device=dev)
        bmins = torch.empty(nb, dtype=x.dtype, device=dev)
        wmins = torch.empty(nb * W, dtype=x.dtype, device=dev)
        tree = torch.empty(2 * M - 1, dtype=x.dtype, device=dev)
        out = torch.empty(n, dtype=torch.int32, device=dev)
        ci = ctypes.c_int
        self._launch(self.function(b"wstlPass1KernelI" + t + b"Li128ELi4E"), nb, 128,
                     [_vp(x.data_ptr()), _vp(out.data_ptr()), ci(n), ci(nb), _vp(leaves.data_ptr()),
                      _vp(bmins.data_ptr()), _vp(wmins.data_ptr())])
        self._launch(self.function(b"wstlFillLeavesKernelI" + t + b"E"), (M + 255) // 256, 256,
                     [_vp(bmins.data_ptr()), _vp(tree.data_ptr()), ci(nb), ci(M - 1), ci(M)])
        level_start, level_size = M // 2 - 1, M // 2
        reduce = self.function(b"wstlReduceLevelKernelI" + t + b"E")
        while level_size > 0:
            self._launch(reduce, (level_size + 255) // 256, 256,
                         [_vp(tree.data_ptr()), ci(level_start), ci(level_size)])
            level_size >>= 1
            level_start = int((level_start - 1) / 2)  # C division: truncates toward zero
        self._launch(self.function(b"wstlPass3KernelI" + t + b"Li128ELi4E"), nb, 128,
                     [_vp(x.data_ptr()), _vp(out.data_ptr()), ci(n), ci(nb), _vp(leaves.data_ptr()),
                      _vp(bmins.data_ptr()), _vp(wmins.data_ptr()), _vp(tree.data_ptr()), ci(M - 1)])
        torch.cuda.synchronize()
        return out

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError("%s failed: CUresult %d" % (what, rc))

    def run(self, x: torch.Tensor, incl: bool) -> torch.Tensor:
        n = x.numel()
        B, W = 512, 16  # BLOCK_SIZE * IPT keys per logical block, 32-key words per block
        nb = (n + B - 1) // B
        M = 1
        while M < nb:
            M <<= 1
        dev = x.device
        unres = torch.empty(nb * W, dtype=torch.int32, device=dev)
        bmins = torch.empty(nb, dtype=torch.int32, device=dev)
        wmins = torch.empty(nb * W, dtype=torch.int32, device=dev)
        tree = torch.empty(2 * M - 1, dtype=torch.int32, device=dev)
        pmin = torch.empty(nb, dtype=torch.int32, device=dev)
        out = torch.empty(n, dtype=torch.int32, device=dev)
        f = self.fn[incl]
        per_sm = ctypes.c_int()
        self._check(self.cu.cuOccupancyMaxActiveBlocksPerMultiprocessor(ctypes.byref(per_sm), f, 128, 0),
                    "cuOccupancyMaxActiveBlocksPerMultiprocessor")
        vals = [_vp(x.data_ptr()), _vp(out.data_ptr()), ctypes.c_int(n), ctypes.c_int(nb), ctypes.c_int(M),
                ctypes.c_int(M - 1), _vp(unres.data_ptr()), _vp(bmins.data_ptr()), _vp(wmins.data_ptr()),
                _vp(tree.data_ptr()), _vp(pmin.data_ptr())]
        self._launch(f, per_sm.value * self.sms, 128, vals, cooperative=True)
        torch.cuda.synchronize()
        return out

    def close(self):
        self.cu.cuModuleUnload(self.mod)


@pytest.fixture(scope="module")
def ref():
    r = ReferenceKernels()
    yield r
    r.close()


def inputs(name, n, rng):
    i = np.arange(n, dtype=np.int64)
    if name == "uniform":
        return rng.integers(0, 1 << 31, n).astype(np.int32)
    if name == "descending":
        return (n - 1 - i).astype(np.int32)
    if name == "ascending":
        return i.astype(np.int32)
    if name == "dup16":
        return rng.integers(0, 16, n).astype(np.int32)
    if name == "sawtooth":
        return (i % 257).astype(np.int32)
    if name == "runs":  # descending runs from random starts (the batch workload's middle shape)
        run = int(rng.integers(1, 4097))
        return (rng.integers(0, 1 << 30) - (i % run) + (i // run) * 7).astype(np.int32)
    return np.full(n, 5, dtype=np.int32)  # all equal


NAMES = ["uniform", "descending", "ascending", "dup16", "sawtooth", "runs", "equal"]
SIZES = [1, 2, 31, 511, 512, 513, 4096, 1_000_003, 1 << 20]


@pytest.mark.parametrize("incl", [False, True], ids=["lt", "le"])
@pytest.mark.parametrize("name", NAMES)
def test_engine_matches_the_reference_kernel(ref, name, incl):
    rng = np.random.default_rng(NAMES.index(name) + 100 * incl)
    with Plan(max(SIZES), torch.int32, inclusive=incl, tuning=None) as plan:
        for n in SIZES:
            x = torch.from_numpy(inputs(name, n, rng)).cuda()
            want = ref.run(x, incl)
            got = plan.run(x)
            plan.check()
            if not torch.equal(got, want):
                bad = int(torch.nonzero(got != want)[0])
                pytest.fail("n=%d: first difference at %d: engine %d, reference kernel %d"
                            % (n, bad, int(got[bad]), int(want[bad])))


@pytest.mark.parametrize("name", ["uniform", "descending", "ascending", "dup16"])
def test_engine_matches_the_reference_kernel_at_2p25(ref, name):
    n = 1 << 25
    x = torch.from_numpy(inputs(name, n, np.random.default_rng(1234))).cuda()
    with Plan(n, torch.int32, tuning=None) as plan:
        got = plan.run(x)
        plan.check()
    assert torch.equal(got, ref.run(x, False))


def float_inputs(name, n, rng):
    if name == "uniform":  # the serving workload's float keys: finite, exact
        return (-1e6 + rng.integers(0, 1 << 24, n) * (2e6 / (1 << 24))).astype(np.float32)
    if name == "normal":
        return rng.standard_normal(n).astype(np.float32)
    if name == "zeros":  # -0.0 and +0.0 compare equal
        return np.where(rng.random(n) < 0.5, -0.0, 0.0).astype(np.float32) + \
            np.where(rng.random(n) < 0.1, rng.standard_normal(n), 0).astype(np.float32)
    return inputs(name, n, rng).astype(np.float32)


FLOAT_NAMES = ["uniform", "normal", "zeros", "descending", "ascending", "dup16", "sawtooth"]


@pytest.mark.parametrize("name", NAMES)
def test_engine_matches_the_reference_wstl_int32(ref, name):
    rng = np.random.default_rng(500 + NAMES.index(name))
    with Plan(max(SIZES), torch.int32, tuning=None) as plan:
        for n in SIZES:
            x = torch.from_numpy(inputs(name, n, rng)).cuda()
            got = plan.run(x)
            plan.check()
            assert torch.equal(got, ref.run_wstl(x)), n


@pytest.mark.parametrize("name", FLOAT_NAMES)
def test_engine_matches_the_reference_wstl_float32(ref, name):
    rng = np.random.default_rng(600 + FLOAT_NAMES.index(name))
    with Plan(1 << 25, torch.float32, tuning=None) as plan:
        for n in SIZES + [1 << 25]:
            x = torch.from_numpy(float_inputs(name, n, rng)).cuda()
            got = plan.run(x)
            plan.check()
            want = ref.run_wstl(x)
            if not torch.equal(got, want):
                bad = int(torch.nonzero(got != want)[0])
                pytest.fail("n=%d: first difference at %d: engine %d, reference WSTL %d"
                            % (n, bad, int(got[bad]), int(want[bad])))
