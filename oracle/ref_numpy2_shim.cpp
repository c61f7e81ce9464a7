// Compatibility shim used ONLY to build the reference CEUpdater as a test oracle.
//
// The reference's cpp/src/ce_updater.cpp (lines 657-658, 671, 951, 968, 977)
// hands a PyObject* to numpy's array accessors.  numpy >= 2 declares those
// accessors as inline functions taking `const PyArrayObject*`, so the file no
// longer compiles as-is.  Rather than editing the reference source, this
// translation unit adds PyObject* overloads of the four accessors and then
// compiles the unmodified reference file through #include.  No behaviour of
// the reference changes: each overload is a pointer cast.
#include <Python.h>
#include "use_numpy.hpp"

static inline int PyArray_NDIM(PyObject *o) { return PyArray_NDIM((const PyArrayObject *)o); }
static inline char *PyArray_BYTES(PyObject *o) { return PyArray_BYTES((const PyArrayObject *)o); }
static inline npy_intp *PyArray_DIMS(PyObject *o) { return PyArray_DIMS((const PyArrayObject *)o); }
static inline npy_intp *PyArray_STRIDES(PyObject *o) { return PyArray_STRIDES((const PyArrayObject *)o); }

#include "ce_updater.cpp"
