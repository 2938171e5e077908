// Host-side packing of a batch of requests (CPython extension module _xr_host).
//
// fill(items, type_map, types_out, x_out) walks the batch's request tuples
// (symbols, positions, total_charge, cell, pbc, initial_charges) once in C: each symbol is looked up in
// type_map (label -> type index) and written to types_out (int32, the batch's atoms in order), and
// positions that are a C-contiguous float64 (n, 3) buffer are copied into x_out (float64, atoms x 3)
// after a finiteness check. A request this cannot take as is (another container or dtype, a label
// missing from the map, a non-finite coordinate, a total charge that is not a finite int or float)
// is left for the Python path, which applies xreac's validation and messages; fill returns the
// indices of those requests. Cells and periodicity are always handled in Python.
//
// guesses(items, addr_out) takes the requests' initial charges: None gives address 0, a C-contiguous
// float64 numpy array of one finite charge per atom gives its data address (valid while the caller
// holds the request; other buffer exporters may not keep their memory after the export ends), and
// anything else is left for the Python checks; it returns the indices of those.
#include <Python.h>

#include <cmath>
#include <cstring>

namespace {

bool finite_number(PyObject* q) {
  if (PyFloat_CheckExact(q)) return std::isfinite(PyFloat_AS_DOUBLE(q));
  return PyLong_CheckExact(q) != 0;
}

// 0: taken; 1: left for Python; -1: a Python error is set
int fill_one(PyObject* item, PyObject* type_map, int* types, double* x, Py_ssize_t natoms) {
  if (!PyTuple_Check(item) || PyTuple_GET_SIZE(item) != 6) return 1;
  PyObject* symbols = PyTuple_GET_ITEM(item, 0);
  PyObject* positions = PyTuple_GET_ITEM(item, 1);
  if (!finite_number(PyTuple_GET_ITEM(item, 2))) return 1;
  if (!PyList_CheckExact(symbols) && !PyTuple_CheckExact(symbols)) return 1;
  PyObject** sym = PySequence_Fast_ITEMS(symbols);
  if (PySequence_Fast_GET_SIZE(symbols) != natoms || natoms == 0) return 1;
  // Labels repeat, usually as the same string objects: a few recently seen objects are matched by
  // identity before the dictionary is asked.
  constexpr int kSeen = 8;
  PyObject* seen[kSeen] = {};
  int seen_type[kSeen] = {};
  int nseen = 0;
  for (Py_ssize_t a = 0; a < natoms; ++a) {
    PyObject* label = sym[a];
    int k = 0;
    while (k < nseen && seen[k] != label) ++k;
    if (k < nseen) {
      types[a] = seen_type[k];
      continue;
    }
    if (!PyUnicode_CheckExact(label)) return 1;
    PyObject* t = PyDict_GetItemWithError(type_map, label);  // borrowed
    if (!t) return PyErr_Occurred() ? -1 : 1;
    const long v = PyLong_AsLong(t);
    if (v == -1 && PyErr_Occurred()) return -1;
    types[a] = (int)v;
    if (nseen < kSeen) {
      seen[nseen] = label;
      seen_type[nseen++] = (int)v;
    }
  }
  Py_buffer view;
  if (PyObject_GetBuffer(positions, &view, PyBUF_C_CONTIGUOUS | PyBUF_FORMAT | PyBUF_ND) != 0) {
    PyErr_Clear();
    return 1;
  }
  int rc = 1;
  if (view.ndim == 2 && view.shape[0] == natoms && view.shape[1] == 3 && view.itemsize == 8 && view.format &&
      std::strcmp(view.format, "d") == 0) {
    const double* src = static_cast<const double*>(view.buf);
    bool ok = true;
    for (Py_ssize_t k = 0; k < 3 * natoms; ++k) ok = ok && std::isfinite(src[k]);
    if (ok) {
      std::memcpy(x, src, sizeof(double) * 3 * (size_t)natoms);
      rc = 0;
    }
  }
  PyBuffer_Release(&view);
  return rc;
}

PyObject* fill(PyObject*, PyObject* args) {
  PyObject *items, *type_map, *types_obj, *x_obj;
  if (!PyArg_ParseTuple(args, "O!O!OO", &PyList_Type, &items, &PyDict_Type, &type_map, &types_obj, &x_obj)) return nullptr;
  Py_buffer tv, xv;
  if (PyObject_GetBuffer(types_obj, &tv, PyBUF_C_CONTIGUOUS | PyBUF_WRITABLE | PyBUF_FORMAT) != 0) return nullptr;
  if (PyObject_GetBuffer(x_obj, &xv, PyBUF_C_CONTIGUOUS | PyBUF_WRITABLE | PyBUF_FORMAT) != 0) {
    PyBuffer_Release(&tv);
    return nullptr;
  }
  PyObject* slow = nullptr;
  const Py_ssize_t total = tv.len / (Py_ssize_t)sizeof(int);
  if (tv.itemsize != 4 || xv.itemsize != 8 || xv.len != 3 * tv.len * 2) {
    PyErr_SetString(PyExc_ValueError, "fill needs int32 types and float64 (atoms, 3) positions");
  } else if ((slow = PyList_New(0)) != nullptr) {
    int* types = static_cast<int*>(tv.buf);
    double* x = static_cast<double*>(xv.buf);
    Py_ssize_t off = 0;
    const Py_ssize_t nitems = PyList_GET_SIZE(items);
    for (Py_ssize_t k = 0; k < nitems; ++k) {
      PyObject* item = PyList_GET_ITEM(items, k);
      if (!PyTuple_Check(item) || PyTuple_GET_SIZE(item) < 1) {
        PyErr_SetString(PyExc_ValueError, "requests must be tuples");
        Py_CLEAR(slow);
        break;
      }
      const Py_ssize_t n = PyObject_Length(PyTuple_GET_ITEM(item, 0));
      if (n < 0 || off + n > total) {
        if (!PyErr_Occurred()) PyErr_SetString(PyExc_ValueError, "atom counts do not match the output size");
        Py_CLEAR(slow);
        break;
      }
      const int rc = fill_one(item, type_map, types + off, x + 3 * off, n);
      if (rc < 0) {
        Py_CLEAR(slow);
        break;
      }
      if (rc == 1) {
        PyObject* idx = PyLong_FromSsize_t(k);
        if (!idx || PyList_Append(slow, idx) != 0) {
          Py_XDECREF(idx);
          Py_CLEAR(slow);
          break;
        }
        Py_DECREF(idx);
      }
      off += n;
    }
  }
  PyBuffer_Release(&tv);
  PyBuffer_Release(&xv);
  return slow;
}

// 0: taken (address in *addr, 0 for None); 1: left for Python
int guess_one(PyObject* item, unsigned long long* addr) {
  *addr = 0;
  if (!PyTuple_Check(item) || PyTuple_GET_SIZE(item) != 6) return 1;
  PyObject* initial = PyTuple_GET_ITEM(item, 5);
  if (initial == Py_None) return 0;
  if (std::strcmp(Py_TYPE(initial)->tp_name, "numpy.ndarray") != 0) return 1;
  const Py_ssize_t n = PyObject_Length(PyTuple_GET_ITEM(item, 0));
  if (n < 0) {
    PyErr_Clear();
    return 1;
  }
  Py_buffer view;
  if (PyObject_GetBuffer(initial, &view, PyBUF_C_CONTIGUOUS | PyBUF_FORMAT | PyBUF_ND) != 0) {
    PyErr_Clear();
    return 1;
  }
  int rc = 1;
  if (view.ndim == 1 && view.shape[0] == n && view.itemsize == 8 && view.format && std::strcmp(view.format, "d") == 0) {
    const double* q = static_cast<const double*>(view.buf);
    bool ok = true;
    for (Py_ssize_t k = 0; k < n; ++k) ok = ok && std::isfinite(q[k]);
    if (ok) {
      *addr = reinterpret_cast<unsigned long long>(view.buf);
      rc = 0;
    }
  }
  PyBuffer_Release(&view);
  return rc;
}

PyObject* guesses(PyObject*, PyObject* args) {
  PyObject *items, *addr_obj;
  if (!PyArg_ParseTuple(args, "O!O", &PyList_Type, &items, &addr_obj)) return nullptr;
  Py_buffer av;
  if (PyObject_GetBuffer(addr_obj, &av, PyBUF_C_CONTIGUOUS | PyBUF_WRITABLE | PyBUF_FORMAT) != 0) return nullptr;
  const Py_ssize_t nitems = PyList_GET_SIZE(items);
  PyObject* slow = nullptr;
  if (av.itemsize != 8 || av.len != 8 * nitems) {
    PyErr_SetString(PyExc_ValueError, "guesses needs one uint64 address per request");
  } else if ((slow = PyList_New(0)) != nullptr) {
    unsigned long long* addr = static_cast<unsigned long long*>(av.buf);
    for (Py_ssize_t k = 0; k < nitems; ++k) {
      if (guess_one(PyList_GET_ITEM(items, k), addr + k) == 0) continue;
      PyObject* idx = PyLong_FromSsize_t(k);
      if (!idx || PyList_Append(slow, idx) != 0) {
        Py_XDECREF(idx);
        Py_CLEAR(slow);
        break;
      }
      Py_DECREF(idx);
    }
  }
  PyBuffer_Release(&av);
  return slow;
}

PyMethodDef methods[] = {
    {"fill", fill, METH_VARARGS, "Pack a batch's symbols and positions; returns the requests left for Python."},
    {"guesses", guesses, METH_VARARGS,
     "Addresses of the requests' initial charges (0 for None); returns the requests left for Python."},
    {nullptr, nullptr, 0, nullptr},
};

PyModuleDef module = {PyModuleDef_HEAD_INIT, "_xr_host", "Host-side batch packing.", -1, methods,
                      nullptr, nullptr, nullptr, nullptr};

}  // namespace

PyMODINIT_FUNC PyInit__xr_host(void) { return PyModule_Create(&module); }
