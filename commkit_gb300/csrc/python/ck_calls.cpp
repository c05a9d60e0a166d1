// ck_calls: the per-call path of compute_llr() and decode() for torch CUDA
// tensors, as a CPython extension over ATen.
//
// One call checks the input tensor, allocates the outputs from ATen's caching
// allocator, takes the current stream and the device guard from c10, calls
// the C ABI of libck_gb300.so through entry points handed over by init(), and
// builds the result objects, without returning to the interpreter in between
// (ctypes argument conversion, Python-level torch.empty calls and the result
// dataclass's __init__ cost more than the launch itself).
//
// The Python layer keeps every rule: it registers an entry (the plan or the
// constellation's device tables) after its general path has served a call of
// that form, and a call this module does not take returns None, after which
// the caller runs the general path, which converts or raises exactly as it
// always did.  It takes: a CUDA strided tensor of the one dtype the kernel
// reads (float32 LLRs, complex64 symbols), contiguous, without conj/neg bits,
// on a device with an entry.  A nonzero status of the C ABI comes back as a
// Python int for the caller to raise with the library's message.
//
// The GIL is held for the whole call, so two host threads never interleave
// the decoder's workspace reset and launch on one stream.

#include <Python.h>

#include <ATen/core/Tensor.h>
#include <ATen/ops/empty.h>
#include <c10/core/TensorImpl.h>
#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>
#include <torch/csrc/autograd/python_variable.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <map>
#include <optional>
#include <utility>

#include "commkit_gb300.h"

namespace {

decltype(&ck_ldpc_decode) g_decode = nullptr;
decltype(&ck_ldpc_workspace_size) g_workspace_size = nullptr;
decltype(&ck_llr_separable_maxlog) g_llr_maxlog = nullptr;
decltype(&ck_llr_separable) g_llr_levels = nullptr;
decltype(&ck_llr_points) g_llr_points = nullptr;
PyTypeObject* g_result_type = nullptr;  // DecodeResult
PyObject* g_empty = nullptr;            // ()
PyObject* g_names[5] = {};              // bits, llrs, valid, iterations, checked

// Decode workspaces per (device, stream), grown on demand.  Work on one
// stream runs in order and the GIL orders the host side, so every plan and
// rule on a stream can share one.  Never destroyed: the process's exit may
// come after the CUDA allocator is gone.
using WorkspaceKey = std::pair<int, cudaStream_t>;
std::map<WorkspaceKey, at::Tensor>* g_workspaces = nullptr;

// Outputs of a decode up to this many bytes share one allocation (one trip
// through the allocator instead of four); larger ones are allocated apiece,
// so keeping one output alive does not keep a large batch's others.
constexpr size_t kSharedOutputBytes = 4u << 20;

constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// The tensor behind `o` if it is a CUDA strided tensor of `type` that the
// kernels can read as it is; nullptr otherwise.
const at::Tensor* plain_cuda(PyObject* o, c10::ScalarType type) {
    if (!THPVariable_Check(o)) return nullptr;
    const at::Tensor& t = THPVariable_Unpack(o);
    if (!t.defined() || !t.is_cuda() || t.layout() != c10::kStrided) return nullptr;
    if (t.scalar_type() != type || t.is_conj() || t.is_neg() || !t.is_contiguous()) return nullptr;
    return &t;
}

// A tensor of `type` and `sizes` over bytes [offset, ...) of `buf`'s storage.
at::Tensor part_of(const at::Tensor& buf, size_t offset, c10::ScalarType type, c10::IntArrayRef sizes) {
    const auto meta = c10::scalarTypeToTypeMeta(type);
    at::Tensor t = at::detail::make_tensor<c10::TensorImpl>(c10::TensorImpl::VIEW, c10::Storage(buf.storage()),
                                                            buf.key_set(), meta);
    auto* impl = t.unsafeGetTensorImpl();
    impl->set_sizes_contiguous(sizes);
    impl->set_storage_offset(static_cast<int64_t>(offset / meta.itemsize()));
    return t;
}

bool as_long(PyObject* o, long long* v) {
    *v = PyLong_AsLongLong(o);
    return !(*v == -1 && PyErr_Occurred());
}

PyObject* bad_call(const char* what) {
    PyErr_SetString(PyExc_TypeError, what);
    return nullptr;
}

// init(decode, workspace_size, llr_separable_maxlog, llr_separable, llr_points, DecodeResult)
PyObject* init(PyObject*, PyObject* const* a, Py_ssize_t na) {
    if (na != 6 || !PyType_Check(a[5])) return bad_call("init(5 entry-point addresses, DecodeResult)");
    void* p[5];
    for (int i = 0; i < 5; ++i) {
        p[i] = PyLong_AsVoidPtr(a[i]);
        if (PyErr_Occurred()) return nullptr;
        if (!p[i]) return bad_call("init(): NULL entry point");
    }
    g_decode = reinterpret_cast<decltype(g_decode)>(p[0]);
    g_workspace_size = reinterpret_cast<decltype(g_workspace_size)>(p[1]);
    g_llr_maxlog = reinterpret_cast<decltype(g_llr_maxlog)>(p[2]);
    g_llr_levels = reinterpret_cast<decltype(g_llr_levels)>(p[3]);
    g_llr_points = reinterpret_cast<decltype(g_llr_points)>(p[4]);
    Py_INCREF(a[5]);
    Py_XSETREF(g_result_type, reinterpret_cast<PyTypeObject*>(a[5]));
    Py_RETURN_NONE;
}

// decode(llrs, entries, call) -> DecodeResult | int status | None
//   entries: list indexed by device of (plan address, n, k) or None;
//   call: (rule, scale, offset, max_iterations, early_stop).
PyObject* decode(PyObject*, PyObject* const* a, Py_ssize_t na) {
    if (na != 3 || !PyList_Check(a[1]) || !PyTuple_Check(a[2]) || PyTuple_GET_SIZE(a[2]) != 5)
        return bad_call("decode(llrs, entries: list, call: 5-tuple)");
    if (!g_decode || !g_result_type) return bad_call("decode(): init() was not called");
    const at::Tensor* tp = plain_cuda(a[0], c10::kFloat);
    if (!tp) Py_RETURN_NONE;
    const at::Tensor& t = *tp;
    const int64_t dim = t.dim();
    if (dim != 1 && dim != 2) Py_RETURN_NONE;
    const int dev = t.get_device();
    if (dev < 0 || dev >= PyList_GET_SIZE(a[1])) Py_RETURN_NONE;
    PyObject* e = PyList_GET_ITEM(a[1], dev);
    if (!PyTuple_Check(e) || PyTuple_GET_SIZE(e) != 3) Py_RETURN_NONE;
    const ck_ldpc_plan* plan = static_cast<const ck_ldpc_plan*>(PyLong_AsVoidPtr(PyTuple_GET_ITEM(e, 0)));
    long long n, k, rule, max_it, early;
    if (PyErr_Occurred() || !as_long(PyTuple_GET_ITEM(e, 1), &n) || !as_long(PyTuple_GET_ITEM(e, 2), &k))
        return nullptr;
    PyObject* c = a[2];
    if (!as_long(PyTuple_GET_ITEM(c, 0), &rule) || !as_long(PyTuple_GET_ITEM(c, 3), &max_it) ||
        !as_long(PyTuple_GET_ITEM(c, 4), &early))
        return nullptr;
    const double scale = PyFloat_AsDouble(PyTuple_GET_ITEM(c, 1));
    const double offset = PyFloat_AsDouble(PyTuple_GET_ITEM(c, 2));
    if (PyErr_Occurred()) return nullptr;
    const auto sizes = t.sizes();
    const int64_t last = sizes[dim - 1];
    if (!plan || n <= 0 || k < 0 || last % n) Py_RETURN_NONE;
    const int64_t C = dim == 1 ? 1 : sizes[0];
    const int64_t nb = last / n;
    const int64_t rows = C * nb;
    if (rows <= 0) Py_RETURN_NONE;

    at::Tensor out, bits, iters, valid, ws;
    cudaStream_t s;
    std::optional<c10::cuda::CUDAGuard> guard;
    try {
        guard.emplace(static_cast<c10::DeviceIndex>(dev));
        s = c10::cuda::getCurrentCUDAStream(static_cast<c10::DeviceIndex>(dev)).stream();
        size_t need = 0;
        const int st = g_workspace_size(plan, rows, static_cast<int32_t>(rule), &need);
        if (st != CK_OK) return PyLong_FromLong(st);
        if (!g_workspaces) g_workspaces = new std::map<WorkspaceKey, at::Tensor>();
        at::Tensor& slot = (*g_workspaces)[WorkspaceKey(dev, s)];
        if (!slot.defined() || static_cast<size_t>(slot.numel()) < need)
            slot = at::empty({static_cast<int64_t>(std::max<size_t>(need, 256))}, t.options().dtype(c10::kByte));
        ws = slot;

        const int64_t lead[1] = {C};
        const c10::IntArrayRef head(lead, dim == 1 ? 0 : 1);
        auto shape = [&](int64_t inner) {
            c10::SmallVector<int64_t, 2> v(head.begin(), head.end());
            v.push_back(inner);
            return v;
        };
        const auto s_llr = shape(nb * n), s_bits = shape(nb * k), s_frame = shape(nb);
        const size_t b_llr = align256(size_t(rows) * size_t(n) * 4), b_it = align256(size_t(rows) * 4),
                     b_valid = align256(size_t(rows)), b_bits = size_t(rows) * size_t(k);
        if (b_llr + b_it + b_valid + b_bits <= kSharedOutputBytes) {
            const at::Tensor buf = at::empty({static_cast<int64_t>(b_llr + b_it + b_valid + b_bits)},
                                             t.options().dtype(c10::kByte));
            out = part_of(buf, 0, c10::kFloat, s_llr);
            iters = part_of(buf, b_llr, c10::kInt, s_frame);
            valid = part_of(buf, b_llr + b_it, c10::kBool, s_frame);
            bits = part_of(buf, b_llr + b_it + b_valid, c10::kChar, s_bits);
        } else {
            out = at::empty(s_llr, t.options());
            iters = at::empty(s_frame, t.options().dtype(c10::kInt));
            valid = at::empty(s_frame, t.options().dtype(c10::kBool));
            bits = at::empty(s_bits, t.options().dtype(c10::kChar));
        }
    } catch (const std::exception&) {
        // An allocation that failed: the general path repeats it and raises
        // torch's own error.
        Py_RETURN_NONE;
    }
    {
        const int st = g_decode(plan, t.const_data_ptr<float>(), out.mutable_data_ptr<float>(), rows,
                                static_cast<int32_t>(n), static_cast<int32_t>(rule), static_cast<float>(scale),
                                static_cast<float>(offset), static_cast<int32_t>(max_it),
                                static_cast<int32_t>(early), iters.mutable_data_ptr<int32_t>(),
                                reinterpret_cast<uint8_t*>(valid.mutable_data_ptr<bool>()),
                                bits.mutable_data_ptr<int8_t>(), static_cast<int32_t>(k), ws.mutable_data_ptr(),
                                static_cast<size_t>(ws.numel()), s);
        if (st != CK_OK) return PyLong_FromLong(st);
    }
    PyObject* r = PyBaseObject_Type.tp_new(g_result_type, g_empty, nullptr);
    if (!r) return nullptr;
    PyObject* vals[5] = {THPVariable_Wrap(std::move(bits)), THPVariable_Wrap(std::move(out)),
                         THPVariable_Wrap(std::move(valid)), THPVariable_Wrap(std::move(iters)), Py_True};
    int bad = 0;
    for (int i = 0; i < 5; ++i) {
        // object.__setattr__: the dataclass is frozen against later changes.
        if (!vals[i] || PyObject_GenericSetAttr(r, g_names[i], vals[i]) < 0) bad = 1;
        if (i < 4) Py_XDECREF(vals[i]);
    }
    if (bad) {
        Py_DECREF(r);
        return nullptr;
    }
    return r;
}

// llr(symbols, noise_var, entries) -> tensor | int status | None
//   entries: list indexed by device of (kind, exact, p0, p1, p2, M, k) or
//   None; kind 0 closed-form max-log (p0/p1 the axis structs), 1 per-axis
//   levels (p0/p1 the axis structs), 2 every point (p0 points, p1 log_pmf,
//   p2 labels).
PyObject* llr(PyObject*, PyObject* const* a, Py_ssize_t na) {
    if (na != 3 || !PyList_Check(a[2])) return bad_call("llr(symbols, noise_var, entries: list)");
    if (!g_llr_maxlog) return bad_call("llr(): init() was not called");
    const at::Tensor* tp = plain_cuda(a[0], c10::kComplexFloat);
    if (!tp) Py_RETURN_NONE;
    const at::Tensor& t = *tp;
    // The noise variance as the general path reads it (float(v), finite,
    // >= 0); anything else goes there to be converted or refused.
    double nv;
    if (PyFloat_Check(a[1])) {
        nv = PyFloat_AS_DOUBLE(a[1]);
    } else if (PyLong_Check(a[1])) {
        nv = PyLong_AsDouble(a[1]);
        if (nv == -1.0 && PyErr_Occurred()) {
            PyErr_Clear();
            Py_RETURN_NONE;
        }
    } else {
        Py_RETURN_NONE;
    }
    if (!std::isfinite(nv) || nv < 0.0) Py_RETURN_NONE;
    const int dev = t.get_device();
    if (dev < 0 || dev >= PyList_GET_SIZE(a[2])) Py_RETURN_NONE;
    PyObject* e = PyList_GET_ITEM(a[2], dev);
    if (!PyTuple_Check(e) || PyTuple_GET_SIZE(e) != 7) Py_RETURN_NONE;
    long long v[7];
    for (int i = 0; i < 7; ++i) {
        v[i] = static_cast<long long>(PyLong_AsSsize_t(PyTuple_GET_ITEM(e, i)));
        if (v[i] == -1 && PyErr_Occurred()) return nullptr;
    }
    const long long kind = v[0], exact = v[1], M = v[5], k = v[6];
    const int64_t n = t.numel();
    if (n >= (int64_t(1) << 31) || k < 1) Py_RETURN_NONE;
    // float32(1 / max(nv, 1e-20)): the double quotient rounded once.
    const float inv_s2 = static_cast<float>(1.0 / std::max(nv, 1e-20));
    at::Tensor out;
    cudaStream_t s;
    std::optional<c10::cuda::CUDAGuard> guard;
    try {
        guard.emplace(static_cast<c10::DeviceIndex>(dev));
        s = c10::cuda::getCurrentCUDAStream(static_cast<c10::DeviceIndex>(dev)).stream();
        if (t.dim() == 0) {
            out = at::empty({k}, t.options().dtype(c10::kFloat));
        } else {
            auto shape = t.sizes().vec();
            shape.back() *= k;
            out = at::empty(shape, t.options().dtype(c10::kFloat));
        }
    } catch (const std::exception&) {
        Py_RETURN_NONE;
    }
    int st;
    {
        const void* x = t.const_data_ptr();
        float* o = out.mutable_data_ptr<float>();
        const auto ptr = [&](int i) { return reinterpret_cast<const void*>(static_cast<uintptr_t>(v[i])); };
        if (kind == 0)
            st = g_llr_maxlog(x, n, static_cast<const ck_axis_maxlog*>(ptr(2)),
                              static_cast<const ck_axis_maxlog*>(ptr(3)), inv_s2, o, s);
        else if (kind == 1)
            st = g_llr_levels(x, n, static_cast<const ck_axis_levels*>(ptr(2)),
                              static_cast<const ck_axis_levels*>(ptr(3)), inv_s2, static_cast<int32_t>(exact), o, s);
        else if (kind == 2)
            st = g_llr_points(x, n, ptr(2), static_cast<const float*>(ptr(3)), static_cast<const int32_t*>(ptr(4)),
                              static_cast<int32_t>(M), static_cast<int32_t>(k), inv_s2, static_cast<int32_t>(exact),
                              o, s);
        else
            Py_RETURN_NONE;
    }
    if (st != CK_OK) return PyLong_FromLong(st);
    return THPVariable_Wrap(std::move(out));
}

// release(): drops the cached decode workspaces (they return to torch's allocator).
PyObject* release(PyObject*, PyObject*) {
    if (g_workspaces) g_workspaces->clear();
    Py_RETURN_NONE;
}

// workspaces(): the (device, stream handle) pairs holding a decode workspace.
PyObject* workspaces(PyObject*, PyObject*) {
    PyObject* out = PyList_New(0);
    if (!out || !g_workspaces) return out;
    for (const auto& kv : *g_workspaces) {
        PyObject* item = Py_BuildValue("(iK)", kv.first.first,
                                       static_cast<unsigned long long>(reinterpret_cast<uintptr_t>(kv.first.second)));
        if (!item || PyList_Append(out, item) < 0) {
            Py_XDECREF(item);
            Py_DECREF(out);
            return nullptr;
        }
        Py_DECREF(item);
    }
    return out;
}

PyMethodDef methods[] = {
    {"init", reinterpret_cast<PyCFunction>(reinterpret_cast<void (*)(void)>(init)), METH_FASTCALL, nullptr},
    {"decode", reinterpret_cast<PyCFunction>(reinterpret_cast<void (*)(void)>(decode)), METH_FASTCALL, nullptr},
    {"llr", reinterpret_cast<PyCFunction>(reinterpret_cast<void (*)(void)>(llr)), METH_FASTCALL, nullptr},
    {"release", release, METH_NOARGS, nullptr},
    {"workspaces", workspaces, METH_NOARGS, nullptr},
    {nullptr, nullptr, 0, nullptr},
};

PyModuleDef module_def = {PyModuleDef_HEAD_INIT, "ck_calls",
                          "Per-call path of compute_llr() and decode() for torch CUDA tensors.", -1, methods};

}  // namespace

PyMODINIT_FUNC PyInit_ck_calls() {
    static const char* names[5] = {"bits", "llrs", "valid", "iterations", "checked"};
    for (int i = 0; i < 5; ++i)
        if (!g_names[i] && !(g_names[i] = PyUnicode_InternFromString(names[i]))) return nullptr;
    if (!g_empty && !(g_empty = PyTuple_New(0))) return nullptr;
    return PyModule_Create(&module_def);
}
