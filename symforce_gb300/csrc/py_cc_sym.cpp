// _cc_sym_gpu: a compiled Python binding of the GPU optimizer shaped like the reference's cc_sym
// Optimizer binding (symforce/pybind/cc_optimizer.cc:29-170): Optimizer(params, problem, name, keys,
// epsilon), .optimize(values, num_iterations, populate_best_linearization) -> OptimizationStats,
// .linearize(values), .keys(), .update_params(params); module functions optimize(params, problem,
// values, epsilon) and default_optimizer_params().
//
// The reference's Optimizer takes a list of sym::Factor (std::functions the GPU cannot call); this
// one takes the same problem as typed factor batches: any object with `key_types` (int sequence),
// `batches` (objects with `kind`, `keys` int32 [count, num_keys] and `consts` float64
// [count, num_consts], C-contiguous buffers) and optionally `num_schur_keys`.  Values are a writable
// C-contiguous float64 buffer of every key's storage in key order, updated in place with the best
// values like Optimizer.optimize(values) updates a cc_sym.Values.  Written against the CPython C API
// (no binding library), built by symforce_gb300/_build.py.
#define PY_SSIZE_T_CLEAN
#include <Python.h>

#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "sfgpu.h"

namespace {

const char* kParamInt[] = {"verbose", "debug_stats", "check_derivatives", "include_jacobians", "debug_checks",
                           "lambda_update_type", "dynamic_lambda_update_p", "use_diagonal_damping",
                           "use_unit_damping", "keep_max_diagonal_damping", "iterations", "enable_bold_updates"};
const char* kParamDouble[] = {"initial_lambda", "lambda_lower_bound", "lambda_upper_bound", "lambda_up_factor",
                              "lambda_down_factor", "dynamic_lambda_update_beta", "dynamic_lambda_update_gamma",
                              "diagonal_damping_min", "early_exit_min_reduction", "early_exit_min_absolute_error"};

int32_t* IntField(sfg_optimizer_params_t& p, const char* n) {
  if (!strcmp(n, "verbose")) return &p.verbose;
  if (!strcmp(n, "debug_stats")) return &p.debug_stats;
  if (!strcmp(n, "check_derivatives")) return &p.check_derivatives;
  if (!strcmp(n, "include_jacobians")) return &p.include_jacobians;
  if (!strcmp(n, "debug_checks")) return &p.debug_checks;
  if (!strcmp(n, "lambda_update_type")) return &p.lambda_update_type;
  if (!strcmp(n, "dynamic_lambda_update_p")) return &p.dynamic_lambda_update_p;
  if (!strcmp(n, "use_diagonal_damping")) return &p.use_diagonal_damping;
  if (!strcmp(n, "use_unit_damping")) return &p.use_unit_damping;
  if (!strcmp(n, "keep_max_diagonal_damping")) return &p.keep_max_diagonal_damping;
  if (!strcmp(n, "iterations")) return &p.iterations;
  return &p.enable_bold_updates;
}
double* DoubleField(sfg_optimizer_params_t& p, const char* n) {
  if (!strcmp(n, "initial_lambda")) return &p.initial_lambda;
  if (!strcmp(n, "lambda_lower_bound")) return &p.lambda_lower_bound;
  if (!strcmp(n, "lambda_upper_bound")) return &p.lambda_upper_bound;
  if (!strcmp(n, "lambda_up_factor")) return &p.lambda_up_factor;
  if (!strcmp(n, "lambda_down_factor")) return &p.lambda_down_factor;
  if (!strcmp(n, "dynamic_lambda_update_beta")) return &p.dynamic_lambda_update_beta;
  if (!strcmp(n, "dynamic_lambda_update_gamma")) return &p.dynamic_lambda_update_gamma;
  if (!strcmp(n, "diagonal_damping_min")) return &p.diagonal_damping_min;
  if (!strcmp(n, "early_exit_min_reduction")) return &p.early_exit_min_reduction;
  return &p.early_exit_min_absolute_error;
}

// A field of a mapping or an attribute of an object (new reference), or null without error.
PyObject* Field(PyObject* o, const char* name) {
  if (!o || o == Py_None) return nullptr;
  PyObject* v = PyMapping_Check(o) && !PyObject_HasAttrString(o, name) ? PyMapping_GetItemString(o, name)
                                                                        : PyObject_GetAttrString(o, name);
  if (!v) PyErr_Clear();
  return v;
}

// optimizer_params_t from a mapping / object with the reference's field names (missing fields keep
// DefaultOptimizerParams, symforce/opt/optimizer.cc:8-56).
bool ParseParams(PyObject* o, sfg_optimizer_params_t* p) {
  sfg_default_optimizer_params(p);
  for (const char* n : kParamInt) {
    PyObject* v = Field(o, n);
    if (!v) continue;
    PyObject* iv = PyObject_GetAttrString(v, "value");  // enum-like objects
    if (!iv) PyErr_Clear();
    const long x = PyLong_AsLong(iv ? iv : v);
    Py_XDECREF(iv);
    Py_DECREF(v);
    if (x == -1 && PyErr_Occurred()) return false;
    *IntField(*p, n) = int32_t(x);
  }
  for (const char* n : kParamDouble) {
    PyObject* v = Field(o, n);
    if (!v) continue;
    const double x = PyFloat_AsDouble(v);
    Py_DECREF(v);
    if (x == -1.0 && PyErr_Occurred()) return false;
    *DoubleField(*p, n) = x;
  }
  return true;
}

PyObject* ParamsDict(const sfg_optimizer_params_t& p0) {
  sfg_optimizer_params_t p = p0;
  PyObject* d = PyDict_New();
  for (const char* n : kParamInt) {
    PyObject* v = PyLong_FromLong(*IntField(p, n));
    PyDict_SetItemString(d, n, v);
    Py_DECREF(v);
  }
  for (const char* n : kParamDouble) {
    PyObject* v = PyFloat_FromDouble(*DoubleField(p, n));
    PyDict_SetItemString(d, n, v);
    Py_DECREF(v);
  }
  return d;
}

bool Fail(int32_t rc) {
  if (rc == SFG_OK) return false;
  PyErr_Format(PyExc_RuntimeError, "sfgpu error %d: %s", int(rc), sfg_last_error());
  return true;
}

// A C-contiguous buffer of the given format ("i": int32, "d": float64).
struct Buffer {
  Py_buffer view{};
  bool ok = false;
  Buffer(PyObject* o, const char* fmt, bool writable) {
    const int flags = PyBUF_C_CONTIGUOUS | PyBUF_FORMAT | (writable ? PyBUF_WRITABLE : 0);
    if (PyObject_GetBuffer(o, &view, flags) != 0) return;
    const char* f = view.format ? view.format : "B";
    if (*f == '<' || *f == '=' || *f == '@') ++f;
    const bool match = (fmt[0] == 'd' && !strcmp(f, "d") && view.itemsize == 8) ||
                       (fmt[0] == 'i' && (!strcmp(f, "i") || !strcmp(f, "l")) && view.itemsize == 4);
    if (!match) {
      PyErr_Format(PyExc_TypeError, "expected a C-contiguous %s buffer", fmt[0] == 'd' ? "float64" : "int32");
      PyBuffer_Release(&view);
      return;
    }
    ok = true;
  }
  ~Buffer() {
    if (ok) PyBuffer_Release(&view);
  }
  Py_ssize_t count() const { return view.len / view.itemsize; }
};

PyObject* Namespace(PyObject* kwargs) {
  PyObject* types = PyImport_ImportModule("types");
  if (!types) return nullptr;
  PyObject* ns_type = PyObject_GetAttrString(types, "SimpleNamespace");
  Py_DECREF(types);
  if (!ns_type) return nullptr;
  PyObject* empty = PyTuple_New(0);
  PyObject* r = PyObject_Call(ns_type, empty, kwargs);
  Py_DECREF(empty);
  Py_DECREF(ns_type);
  return r;
}

PyObject* DoubleArray(const double* v, size_t n) {
  PyObject* mod = PyImport_ImportModule("array");
  if (!mod) return nullptr;
  PyObject* bytes = PyBytes_FromStringAndSize(reinterpret_cast<const char*>(v), Py_ssize_t(n * sizeof(double)));
  PyObject* r = PyObject_CallMethod(mod, "array", "sO", "d", bytes);
  Py_DECREF(bytes);
  Py_DECREF(mod);
  return r;
}
PyObject* IntArray(const int32_t* v, size_t n) {
  PyObject* mod = PyImport_ImportModule("array");
  if (!mod) return nullptr;
  PyObject* bytes = PyBytes_FromStringAndSize(reinterpret_cast<const char*>(v), Py_ssize_t(n * sizeof(int32_t)));
  PyObject* r = PyObject_CallMethod(mod, "array", "sO", "i", bytes);
  Py_DECREF(bytes);
  Py_DECREF(mod);
  return r;
}

// ---- Optimizer type ---------------------------------------------------------------------------
struct PyOptimizer {
  PyObject_HEAD
  sfg_handle* h;
  sfg_optimizer_params_t params;
  int64_t storage_dim, tangent_dim, residual_dim;
  int32_t num_keys;
  PyObject* name;
};

void OptimizerDealloc(PyOptimizer* self) {
  if (self->h) sfg_destroy(self->h);
  Py_XDECREF(self->name);
  Py_TYPE(self)->tp_free(reinterpret_cast<PyObject*>(self));
}

int OptimizerInit(PyOptimizer* self, PyObject* args, PyObject* kwds) {
  static const char* kw[] = {"params", "problem", "name", "keys", "epsilon", "form", nullptr};
  PyObject *params = nullptr, *problem = nullptr, *keys = Py_None, *form = Py_None;
  const char* name = "sym::Optimize";
  double epsilon = 10.0 * 2.220446049250313e-16;  // sym::kDefaultEpsilon<double>
  if (!PyArg_ParseTupleAndKeywords(args, kwds, "OO|sOdO", const_cast<char**>(kw), &params, &problem, &name,
                                   &keys, &epsilon, &form))
    return -1;
  if (!ParseParams(params, &self->params)) return -1;
  // key types
  PyObject* kt = Field(problem, "key_types");
  PyObject* batches = Field(problem, "batches");
  if (!kt || !batches) {
    Py_XDECREF(kt);
    Py_XDECREF(batches);
    PyErr_SetString(PyExc_TypeError, "problem needs key_types and batches");
    return -1;
  }
  std::vector<int32_t> key_types;
  {
    PyObject* seq = PySequence_Fast(kt, "key_types must be a sequence");
    Py_DECREF(kt);
    if (!seq) {
      Py_DECREF(batches);
      return -1;
    }
    for (Py_ssize_t i = 0; i < PySequence_Fast_GET_SIZE(seq); ++i)
      key_types.push_back(int32_t(PyLong_AsLong(PySequence_Fast_GET_ITEM(seq, i))));
    Py_DECREF(seq);
    if (PyErr_Occurred()) {
      Py_DECREF(batches);
      return -1;
    }
  }
  self->num_keys = int32_t(key_types.size());
  if (keys != Py_None && PyObject_IsTrue(keys)) {
    PyObject* seq = PySequence_Fast(keys, "keys must be a sequence");
    bool all = seq && PySequence_Fast_GET_SIZE(seq) == Py_ssize_t(key_types.size());
    for (Py_ssize_t i = 0; all && i < PySequence_Fast_GET_SIZE(seq); ++i)
      all = PyLong_AsLong(PySequence_Fast_GET_ITEM(seq, i)) == long(i);
    Py_XDECREF(seq);
    if (!all) {
      Py_DECREF(batches);
      if (!PyErr_Occurred())
        PyErr_SetString(PyExc_ValueError, "keys: the device optimizer optimizes every key of the problem in order");
      return -1;
    }
  }
  // batches: keep the buffers alive until sfg_create has copied them
  PyObject* bseq = PySequence_Fast(batches, "batches must be a sequence");
  Py_DECREF(batches);
  if (!bseq) return -1;
  const Py_ssize_t nb = PySequence_Fast_GET_SIZE(bseq);
  std::vector<sfg_factor_batch_t> fb(size_t(nb > 0 ? nb : 1));
  std::vector<std::unique_ptr<Buffer>> bufs;
  for (Py_ssize_t b = 0; b < nb; ++b) {
    PyObject* bo = PySequence_Fast_GET_ITEM(bseq, b);
    PyObject *kind = Field(bo, "kind"), *bk = Field(bo, "keys"), *bc = Field(bo, "consts");
    if (!kind || !bk || !bc) {
      Py_XDECREF(kind);
      Py_XDECREF(bk);
      Py_XDECREF(bc);
      Py_DECREF(bseq);
      PyErr_SetString(PyExc_TypeError, "each batch needs kind, keys and consts");
      return -1;
    }
    int32_t nk = 0, nc = 0, rd = 0;
    const int32_t k = int32_t(PyLong_AsLong(kind));
    Py_DECREF(kind);
    bufs.emplace_back(new Buffer(bk, "i", false));
    bufs.emplace_back(new Buffer(bc, "d", false));
    Py_DECREF(bk);
    Py_DECREF(bc);
    if (!bufs[bufs.size() - 2]->ok || !bufs.back()->ok || Fail(sfg_factor_dims(k, &nk, &nc, &rd))) {
      Py_DECREF(bseq);
      return -1;
    }
    const Py_ssize_t count = nk ? bufs[bufs.size() - 2]->count() / nk : 0;
    fb[size_t(b)] = {k, int32_t(count), static_cast<const int32_t*>(bufs[bufs.size() - 2]->view.buf),
                     static_cast<const double*>(bufs.back()->view.buf)};
  }
  Py_DECREF(bseq);
  int32_t num_schur = 0;
  if (PyObject* ns = Field(problem, "num_schur_keys")) {
    num_schur = int32_t(PyLong_AsLong(ns));
    Py_DECREF(ns);
  }
  sfg_problem_t p{self->num_keys, key_types.data(), int32_t(nb), fb.data(), num_schur};
  sfg_form_params_t fp;
  sfg_default_form_params(&fp);
  fp.epsilon = epsilon;
  fp.linear_solver = num_schur > 0 ? SFG_LINEAR_SOLVER_SCHUR : SFG_LINEAR_SOLVER_SPARSE_LDLT;
  const char* form_int[] = {"precision",    "linear_solver", "ordering",   "device",
                            "refine_steps", "pcg_max_iters", "pcg_coarse", "pcg_band"};
  int32_t* form_dst[] = {&fp.precision,    &fp.linear_solver, &fp.ordering,   &fp.device,
                         &fp.refine_steps, &fp.pcg_max_iters, &fp.pcg_coarse, &fp.pcg_band};
  for (int i = 0; i < 8; ++i)
    if (PyObject* v = Field(form, form_int[i])) {
      *form_dst[i] = int32_t(PyLong_AsLong(v));
      Py_DECREF(v);
    }
  if (PyObject* v = Field(form, "pcg_tol")) {
    fp.pcg_tol = PyFloat_AsDouble(v);
    Py_DECREF(v);
  }
  if (PyErr_Occurred()) return -1;
  int32_t rc;
  Py_BEGIN_ALLOW_THREADS
  rc = sfg_create(&p, &fp, &self->h);
  Py_END_ALLOW_THREADS
  if (Fail(rc)) return -1;
  if (Fail(sfg_storage_dim(self->h, &self->storage_dim, &self->tangent_dim, &self->residual_dim))) return -1;
  self->name = PyUnicode_FromString(name);
  return 0;
}

PyObject* LinearizeImpl(PyOptimizer* self) {
  std::vector<double> res(size_t(self->residual_dim)), rhs(size_t(self->tangent_dim));
  double err = 0;
  int32_t rc;
  Py_BEGIN_ALLOW_THREADS
  rc = sfg_linearize(self->h, res.data(), rhs.data(), &err);
  Py_END_ALLOW_THREADS
  if (Fail(rc)) return nullptr;
  int64_t nnz = 0;
  if (Fail(sfg_hessian_lower(self->h, &nnz, nullptr, nullptr, nullptr))) return nullptr;
  std::vector<int32_t> cp(size_t(self->tangent_dim) + 1), ri(static_cast<size_t>(nnz));
  std::vector<double> hv(static_cast<size_t>(nnz));
  if (Fail(sfg_hessian_lower(self->h, &nnz, cp.data(), ri.data(), hv.data()))) return nullptr;
  PyObject* kw = PyDict_New();
  PyObject* items[][2] = {{PyUnicode_FromString("residual"), DoubleArray(res.data(), res.size())},
                          {PyUnicode_FromString("rhs"), DoubleArray(rhs.data(), rhs.size())},
                          {PyUnicode_FromString("error"), PyFloat_FromDouble(err)},
                          {PyUnicode_FromString("hessian_col_ptr"), IntArray(cp.data(), cp.size())},
                          {PyUnicode_FromString("hessian_row_idx"), IntArray(ri.data(), ri.size())},
                          {PyUnicode_FromString("hessian_values"), DoubleArray(hv.data(), hv.size())}};
  for (auto& it : items) {
    if (!it[1]) {
      Py_DECREF(kw);
      return nullptr;
    }
    PyDict_SetItem(kw, it[0], it[1]);
    Py_DECREF(it[0]);
    Py_DECREF(it[1]);
  }
  PyObject* r = Namespace(kw);
  Py_DECREF(kw);
  return r;
}

PyObject* OptimizerOptimize(PyOptimizer* self, PyObject* args, PyObject* kwds) {
  static const char* kw[] = {"values", "num_iterations", "populate_best_linearization", nullptr};
  PyObject* values;
  int num_iterations = -1, populate = 0;
  if (!PyArg_ParseTupleAndKeywords(args, kwds, "O|ip", const_cast<char**>(kw), &values, &num_iterations, &populate))
    return nullptr;
  Buffer vb(values, "d", true);
  if (!vb.ok) return nullptr;
  if (vb.count() != self->storage_dim) {
    PyErr_Format(PyExc_ValueError, "values has %zd entries, the problem's storage is %lld", vb.count(),
                 (long long)self->storage_dim);
    return nullptr;
  }
  double* v = static_cast<double*>(vb.view.buf);
  const int cap = (num_iterations < 0 ? self->params.iterations : num_iterations) + 1;
  std::vector<sfg_iteration_t> recs(size_t(cap > 1 ? cap : 1));
  sfg_stats_t st{recs.data(), int32_t(recs.size()), 0, 0, 0, 0, 0, 0.0};
  int32_t rc;
  Py_BEGIN_ALLOW_THREADS
  rc = sfg_set_values(self->h, v, self->storage_dim);
  if (rc == SFG_OK) rc = sfg_optimize(self->h, &self->params, num_iterations, &st);
  if (rc == SFG_OK) rc = sfg_get_values(self->h, v, self->storage_dim);
  Py_END_ALLOW_THREADS
  if (Fail(rc)) return nullptr;
  PyObject* its = PyList_New(st.num_iterations);
  for (int i = 0; i < st.num_iterations; ++i) {
    const sfg_iteration_t& r = recs[size_t(i)];
    PyObject* d = Py_BuildValue("{s:i,s:d,s:d,s:d,s:d,s:d,s:O}", "iteration", r.iteration, "current_lambda",
                                r.current_lambda, "new_error", r.new_error, "new_error_linear", r.new_error_linear,
                                "relative_reduction", r.relative_reduction, "update_angle_change",
                                r.update_angle_change, "update_accepted", r.update_accepted ? Py_True : Py_False);
    PyObject* ns = d ? Namespace(d) : nullptr;
    Py_XDECREF(d);
    if (!ns) {
      Py_DECREF(its);
      return nullptr;
    }
    PyList_SET_ITEM(its, i, ns);
  }
  PyObject* best_lin = Py_None;
  Py_INCREF(Py_None);
  if (populate) {
    Py_DECREF(Py_None);
    best_lin = LinearizeImpl(self);  // at the best values the call left on the device
    if (!best_lin) {
      Py_DECREF(its);
      return nullptr;
    }
  }
  PyObject* d = Py_BuildValue("{s:N,s:i,s:i,s:i,s:N,s:d}", "iterations", its, "best_index", st.best_index, "status",
                              st.status, "failure_reason", st.failure_reason, "best_linearization", best_lin,
                              "device_ms", st.device_ms);
  if (!d) return nullptr;
  PyObject* r = Namespace(d);
  Py_DECREF(d);
  return r;
}

PyObject* OptimizerLinearize(PyOptimizer* self, PyObject* args, PyObject* kwds) {
  static const char* kw[] = {"values", nullptr};
  PyObject* values;
  if (!PyArg_ParseTupleAndKeywords(args, kwds, "O", const_cast<char**>(kw), &values)) return nullptr;
  Buffer vb(values, "d", false);
  if (!vb.ok) return nullptr;
  if (vb.count() != self->storage_dim) {
    PyErr_SetString(PyExc_ValueError, "values size does not match the problem's storage");
    return nullptr;
  }
  if (Fail(sfg_set_values(self->h, static_cast<const double*>(vb.view.buf), self->storage_dim))) return nullptr;
  return LinearizeImpl(self);
}

PyObject* OptimizerKeys(PyOptimizer* self, PyObject*) {
  PyObject* l = PyList_New(self->num_keys);
  for (int32_t i = 0; i < self->num_keys; ++i) PyList_SET_ITEM(l, i, PyLong_FromLong(i));
  return l;
}

PyObject* OptimizerUpdateParams(PyOptimizer* self, PyObject* args, PyObject* kwds) {
  static const char* kw[] = {"params", nullptr};
  PyObject* params;
  if (!PyArg_ParseTupleAndKeywords(args, kwds, "O", const_cast<char**>(kw), &params)) return nullptr;
  sfg_optimizer_params_t p;
  if (!ParseParams(params, &p)) return nullptr;
  self->params = p;
  Py_RETURN_NONE;
}

PyObject* OptimizerParams(PyOptimizer* self, PyObject*) { return ParamsDict(self->params); }

PyMethodDef kOptimizerMethods[] = {
    {"optimize", reinterpret_cast<PyCFunction>(reinterpret_cast<void (*)(void)>(OptimizerOptimize)),
     METH_VARARGS | METH_KEYWORDS,
     "optimize(values, num_iterations=-1, populate_best_linearization=False) -> OptimizationStats.\n"
     "Runs the Levenberg-Marquardt loop on the GPU and updates `values` in place with the best values."},
    {"linearize", reinterpret_cast<PyCFunction>(reinterpret_cast<void (*)(void)>(OptimizerLinearize)),
     METH_VARARGS | METH_KEYWORDS, "Linearize the problem around the given values."},
    {"keys", reinterpret_cast<PyCFunction>(OptimizerKeys), METH_NOARGS, "Get the optimized keys (indices)."},
    {"update_params", reinterpret_cast<PyCFunction>(reinterpret_cast<void (*)(void)>(OptimizerUpdateParams)),
     METH_VARARGS | METH_KEYWORDS, "Update the optimizer params."},
    {"params", reinterpret_cast<PyCFunction>(OptimizerParams), METH_NOARGS, "The optimizer params (dict)."},
    {nullptr, nullptr, 0, nullptr}};

PyTypeObject kOptimizerType = {PyVarObject_HEAD_INIT(nullptr, 0)};

PyObject* ModuleDefaultParams(PyObject*, PyObject*) {
  sfg_optimizer_params_t p;
  sfg_default_optimizer_params(&p);
  return ParamsDict(p);
}

PyObject* ModuleOptimize(PyObject*, PyObject* args, PyObject* kwds) {
  static const char* kw[] = {"params", "problem", "values", "epsilon", nullptr};
  PyObject *params, *problem, *values;
  double epsilon = 10.0 * 2.220446049250313e-16;
  if (!PyArg_ParseTupleAndKeywords(args, kwds, "OOO|d", const_cast<char**>(kw), &params, &problem, &values,
                                   &epsilon))
    return nullptr;
  PyObject* ctor_args = Py_BuildValue("(OO)", params, problem);
  PyObject* ctor_kw = Py_BuildValue("{s:d}", "epsilon", epsilon);
  PyObject* opt = PyObject_Call(reinterpret_cast<PyObject*>(&kOptimizerType), ctor_args, ctor_kw);
  Py_DECREF(ctor_args);
  Py_DECREF(ctor_kw);
  if (!opt) return nullptr;
  PyObject* r = PyObject_CallMethod(opt, "optimize", "O", values);
  Py_DECREF(opt);
  return r;
}

PyMethodDef kModuleMethods[] = {
    {"default_optimizer_params", ModuleDefaultParams, METH_NOARGS,
     "Sensible default parameters for Optimizer (sym::DefaultOptimizerParams)."},
    {"optimize", reinterpret_cast<PyCFunction>(reinterpret_cast<void (*)(void)>(ModuleOptimize)),
     METH_VARARGS | METH_KEYWORDS, "Simple wrapper to make optimization one function call."},
    {nullptr, nullptr, 0, nullptr}};

PyModuleDef kModule = {PyModuleDef_HEAD_INIT, "_cc_sym_gpu",
                       "GPU Levenberg-Marquardt optimizer with the reference cc_sym Optimizer's shape.", -1,
                       kModuleMethods};

}  // namespace

PyMODINIT_FUNC PyInit__cc_sym_gpu(void) {
  kOptimizerType.tp_name = "_cc_sym_gpu.Optimizer";
  kOptimizerType.tp_basicsize = sizeof(PyOptimizer);
  kOptimizerType.tp_flags = Py_TPFLAGS_DEFAULT;
  kOptimizerType.tp_doc =
      "Optimizer(params, problem, name='sym::Optimize', keys=None, epsilon=kDefaultEpsilon, form=None): "
      "create once, optimize many (symforce/pybind/cc_optimizer.cc:29-170), on the GPU.";
  kOptimizerType.tp_new = PyType_GenericNew;
  kOptimizerType.tp_init = reinterpret_cast<initproc>(OptimizerInit);
  kOptimizerType.tp_dealloc = reinterpret_cast<destructor>(OptimizerDealloc);
  kOptimizerType.tp_methods = kOptimizerMethods;
  if (PyType_Ready(&kOptimizerType) < 0) return nullptr;
  PyObject* m = PyModule_Create(&kModule);
  if (!m) return nullptr;
  Py_INCREF(&kOptimizerType);
  if (PyModule_AddObject(m, "Optimizer", reinterpret_cast<PyObject*>(&kOptimizerType)) < 0) {
    Py_DECREF(&kOptimizerType);
    Py_DECREF(m);
    return nullptr;
  }
  return m;
}
