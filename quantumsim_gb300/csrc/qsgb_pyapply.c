/*
 * CPython entry point of the per-call apply path: one C call per
 * PauliVectorGB300.apply_ptm with a host PTM.  Through ctypes the same call
 * spends ~4 us converting its 16 arguments and the Python glue around it
 * several more, which is most of a small state's apply_ptm (the reference
 * spends ~36 us of host time per call in PyCUDA,
 * quantumsim/pauli_vectors/cuda.py:151-277).
 *
 * The module links nothing: the library's qsgb_apply_ptm1/2 addresses, the
 * current-stream and status-word lookups, torch.empty and the device
 * constructor are handed over once (set_entry_points).  The output tensor is
 * torch.empty(shape, dtype=pv.dtype, device=<the device of pv>), the device
 * object made once per device index.  The library call runs with the GIL released, as a ctypes call
 * does (a first call of a PTM pattern compiles its kernel).
 *
 * apply(pv, ptm, plan, arith[, out]) -> the output tensor, or an int: the
 * library's status code when the call did not succeed, or NOT_F64_CONTIGUOUS
 * when `ptm` is not a C-contiguous float64 buffer (the caller converts it and
 * calls again).  `plan` is (output shape, two qudits?, sizes, layout flags,
 * dtype code) as built by quantumsim_gb300.ops.eager_plan.  `out` (optional,
 * None for a new tensor) is a contiguous tensor of the output shape, dtype
 * and device that the caller owns and no longer reads, such as the state
 * buffer two applications back: writing into it saves the allocation.
 */
#define PY_SSIZE_T_CLEAN
#include <Python.h>
#include <stdint.h>

typedef int (*apply1_fn)(const void*, void*, const double*, int64_t, int64_t, int64_t, int64_t, int, int, int,
                         int64_t, unsigned*, void*);
typedef int (*apply2_fn)(const void*, void*, const double*, int64_t, int64_t, int64_t, int64_t, int64_t, int64_t,
                         int64_t, int, int, int, int64_t, unsigned*, void*);

#define MAX_DEVICES 64
#define NOT_F64_CONTIGUOUS (-1000)

static apply1_fn g_apply1 = NULL;
static apply2_fn g_apply2 = NULL;
static PyObject* g_raw_stream = NULL; /* callable(device index) -> stream handle (int) */
static PyObject* g_status_ptr = NULL; /* callable(device index) -> status word address */
static unsigned long long g_status[MAX_DEVICES];
static PyObject* g_empty = NULL;       /* torch.empty */
static PyObject* g_device_of = NULL;   /* callable(device index) -> torch.device */
static PyObject* g_dev_obj[MAX_DEVICES];
static PyObject* g_empty_kw = NULL;    /* ("dtype", "device") */
static PyObject* s_data_ptr = NULL;
static PyObject* s_get_device = NULL;
static PyObject* s_dtype = NULL;
static PyObject* s_device = NULL;

static PyObject* set_entry_points(PyObject* self, PyObject* args) {
  unsigned long long a1, a2;
  PyObject *rs, *sp, *em, *dv;
  (void)self;
  if (!PyArg_ParseTuple(args, "KKOOOO", &a1, &a2, &rs, &sp, &em, &dv)) return NULL;
  if (!a1 || !a2 || !PyCallable_Check(rs) || !PyCallable_Check(sp) || !PyCallable_Check(em) ||
      !PyCallable_Check(dv)) {
    PyErr_SetString(PyExc_ValueError, "set_entry_points: null address or non-callable lookup");
    return NULL;
  }
  Py_INCREF(em);
  Py_XDECREF(g_empty);
  g_empty = em;
  Py_INCREF(dv);
  Py_XDECREF(g_device_of);
  g_device_of = dv;
  for (int i = 0; i < MAX_DEVICES; ++i) Py_CLEAR(g_dev_obj[i]);
  g_apply1 = (apply1_fn)(uintptr_t)a1;
  g_apply2 = (apply2_fn)(uintptr_t)a2;
  Py_XINCREF(rs);
  Py_XDECREF(g_raw_stream);
  g_raw_stream = rs;
  Py_XINCREF(sp);
  Py_XDECREF(g_status_ptr);
  g_status_ptr = sp;
  for (int i = 0; i < MAX_DEVICES; ++i) g_status[i] = 0;
  Py_RETURN_NONE;
}

static int as_u64(PyObject* o, unsigned long long* v) {
  if (!o) return -1;
  *v = PyLong_AsUnsignedLongLong(o);
  Py_DECREF(o);
  return (*v == (unsigned long long)-1 && PyErr_Occurred()) ? -1 : 0;
}

static PyObject* apply(PyObject* self, PyObject* const* args, Py_ssize_t nargs) {
  (void)self;
  if (nargs != 4 && nargs != 5) {
    PyErr_SetString(PyExc_TypeError, "apply(pv, ptm, plan, arith[, out])");
    return NULL;
  }
  PyObject* given = (nargs == 5 && args[4] != Py_None) ? args[4] : NULL;
  if (!g_apply1 || !g_apply2 || !g_empty) {
    PyErr_SetString(PyExc_RuntimeError, "apply: set_entry_points was not called");
    return NULL;
  }
  PyObject *pv = args[0], *ptm = args[1], *plan = args[2];
  const int arith = (int)PyLong_AsLong(args[3]);
  if (arith == -1 && PyErr_Occurred()) return NULL;
  if (!PyTuple_Check(plan) || PyTuple_GET_SIZE(plan) != 5) {
    PyErr_SetString(PyExc_TypeError, "apply: plan must be a 5-tuple");
    return NULL;
  }
  PyObject* shape = PyTuple_GET_ITEM(plan, 0);
  const int two = PyObject_IsTrue(PyTuple_GET_ITEM(plan, 1));
  PyObject* sizes = PyTuple_GET_ITEM(plan, 2);
  const int flags = (int)PyLong_AsLong(PyTuple_GET_ITEM(plan, 3));
  const int code = (int)PyLong_AsLong(PyTuple_GET_ITEM(plan, 4));
  if (two < 0 || PyErr_Occurred()) return NULL;
  const Py_ssize_t nsz = two ? 7 : 4;
  if (!PyTuple_Check(sizes) || PyTuple_GET_SIZE(sizes) != nsz || !PyTuple_Check(shape)) {
    PyErr_SetString(PyExc_TypeError, "apply: malformed plan");
    return NULL;
  }
  int64_t sz[7];
  for (Py_ssize_t i = 0; i < nsz; ++i) {
    sz[i] = (int64_t)PyLong_AsLongLong(PyTuple_GET_ITEM(sizes, i));
    if (sz[i] == -1 && PyErr_Occurred()) return NULL;
  }

  /* device, stream and status word */
  PyObject* dev_obj = PyObject_CallMethodNoArgs(pv, s_get_device);
  if (!dev_obj) return NULL;
  const long dev = PyLong_AsLong(dev_obj);
  if (dev == -1 && PyErr_Occurred()) {
    Py_DECREF(dev_obj);
    return NULL;
  }
  if (dev < 0 || dev >= MAX_DEVICES) {
    Py_DECREF(dev_obj);
    PyErr_SetString(PyExc_ValueError, "apply: the state is not on a CUDA device");
    return NULL;
  }
  if (!g_dev_obj[dev]) {
    g_dev_obj[dev] = PyObject_CallOneArg(g_device_of, dev_obj);
    if (!g_dev_obj[dev]) {
      Py_DECREF(dev_obj);
      return NULL;
    }
  }
  unsigned long long stream = 0, status = g_status[dev];
  if (as_u64(PyObject_CallOneArg(g_raw_stream, dev_obj), &stream) < 0) {
    Py_DECREF(dev_obj);
    return NULL;
  }
  if (!status) {
    if (as_u64(PyObject_CallOneArg(g_status_ptr, dev_obj), &status) < 0) {
      Py_DECREF(dev_obj);
      return NULL;
    }
    g_status[dev] = status;
  }
  Py_DECREF(dev_obj);

  /* input and output storage */
  unsigned long long in_ptr = 0, out_ptr = 0;
  if (as_u64(PyObject_CallMethodNoArgs(pv, s_data_ptr), &in_ptr) < 0) return NULL;
  PyObject* out;
  if (given) {
    Py_INCREF(given);
    out = given;
  } else {
    PyObject* kw[3];
    kw[0] = shape;
    kw[1] = PyObject_GetAttr(pv, s_dtype);
    kw[2] = g_dev_obj[dev];
    out = kw[1] ? PyObject_Vectorcall(g_empty, kw, 1, g_empty_kw) : NULL;
    Py_XDECREF(kw[1]);
    if (!out) return NULL;
  }
  for (Py_ssize_t i = 0; i < PyTuple_GET_SIZE(shape); ++i)
    if (PyLong_AsLongLong(PyTuple_GET_ITEM(shape, i)) == 0) return out; /* empty result */
  if (PyErr_Occurred() || as_u64(PyObject_CallMethodNoArgs(out, s_data_ptr), &out_ptr) < 0) {
    Py_DECREF(out);
    return NULL;
  }

  Py_buffer view;
  if (PyObject_GetBuffer(ptm, &view, PyBUF_C_CONTIGUOUS | PyBUF_FORMAT) < 0) {
    PyErr_Clear();
    Py_DECREF(out);
    return PyLong_FromLong(NOT_F64_CONTIGUOUS);
  }
  const char* f = view.format ? view.format : "B";
  if (*f == '<' || *f == '@' || *f == '=') ++f;
  if (view.itemsize != (Py_ssize_t)sizeof(double) || f[0] != 'd' || f[1] != 0 ||
      view.len < (Py_ssize_t)sizeof(double)) {
    PyBuffer_Release(&view);
    Py_DECREF(out);
    return PyLong_FromLong(NOT_F64_CONTIGUOUS);
  }
  int st;
  const void* in = (const void*)(uintptr_t)in_ptr;
  void* o = (void*)(uintptr_t)out_ptr;
  const double* p = (const double*)view.buf;
  unsigned* stp = (unsigned*)(uintptr_t)status;
  void* s = (void*)(uintptr_t)stream;
  Py_BEGIN_ALLOW_THREADS
  if (two)
    st = g_apply2(in, o, p, sz[0], sz[1], sz[2], sz[3], sz[4], sz[5], sz[6], flags, code, arith, 0, stp, s);
  else
    st = g_apply1(in, o, p, sz[0], sz[1], sz[2], sz[3], flags, code, arith, 0, stp, s);
  Py_END_ALLOW_THREADS
  PyBuffer_Release(&view);
  if (st != 0) {
    Py_DECREF(out);
    return PyLong_FromLong(st);
  }
  return out;
}

static PyMethodDef methods[] = {
    {"set_entry_points", set_entry_points, METH_VARARGS,
     "set_entry_points(apply1_addr, apply2_addr, raw_stream, status_ptr, empty, device_of)"},
    {"apply", (PyCFunction)(void (*)(void))apply, METH_FASTCALL,
     "apply(pv, ptm, plan, arith[, out]) -> tensor, or the status code"},
    {NULL, NULL, 0, NULL}};

static struct PyModuleDef module = {PyModuleDef_HEAD_INIT, "_qsgb_pyapply", NULL, -1, methods,
                                    NULL,                  NULL,            NULL, NULL};

PyMODINIT_FUNC PyInit__qsgb_pyapply(void) {
  s_data_ptr = PyUnicode_InternFromString("data_ptr");
  s_get_device = PyUnicode_InternFromString("get_device");
  s_dtype = PyUnicode_InternFromString("dtype");
  s_device = PyUnicode_InternFromString("device");
  if (!s_data_ptr || !s_get_device || !s_dtype || !s_device) return NULL;
  for (int i = 0; i < MAX_DEVICES; ++i) g_dev_obj[i] = NULL;
  g_empty_kw = PyTuple_Pack(2, s_dtype, s_device);
  if (!g_empty_kw) return NULL;
  PyObject* m = PyModule_Create(&module);
  if (m && PyModule_AddIntConstant(m, "NOT_F64_CONTIGUOUS", NOT_F64_CONTIGUOUS) < 0) {
    Py_DECREF(m);
    return NULL;
  }
  return m;
}
