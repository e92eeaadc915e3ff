"""Backend selector mirroring simwave's ``Compiler`` (compiler.py:6-229).

The reference JIT-compiles one C/CUDA source per (dimension, density,
precision) and returns the path of a shared object exporting ``forward``.
Here the language ``'cuda_sm100a'`` (alias ``'cuda_sm103a'``) selects the
prebuilt sm_103a library: ``compile`` returns the path of the variant's shim,
which exports the same ``forward`` symbol. The CPU and OpenMP/OpenACC
languages of the reference are served by the reference package itself.
"""
from . import _lib

LANGUAGES = ('cuda_sm100a', 'cuda_sm103a')


class Compiler:
    """Parameters mirror the reference; ``cc``/``cflags``/``cfile`` are kept
    for API compatibility and validated the same way, but the library is
    built once by ``simwave_gb300.build`` with nvcc for sm_103a."""

    def __init__(self, cc='nvcc', language='cuda_sm100a', cflags=None,
                 cfile=None):
        self.cc = cc
        self.language = language
        self.cflags = cflags
        self.cfile = cfile

    @property
    def cc(self):
        return self._cc

    @cc.setter
    def cc(self, value):
        if not isinstance(value, str):
            raise TypeError("Compiler.cc attribute must be str.")
        self._cc = value

    @property
    def language(self):
        return self._language

    @language.setter
    def language(self, value):
        if not isinstance(value, str):
            raise TypeError("Compiler.language attribute must be str.")
        if value not in LANGUAGES:
            raise ValueError(
                "Compiler.language {} not implemented.".format(value))
        self._language = value

    @property
    def cflags(self):
        return self._cflags

    @cflags.setter
    def cflags(self, value):
        if value is None:
            value = '-O3 -lineinfo -gencode arch=compute_103a,code=sm_103a'
        if not isinstance(value, str):
            raise TypeError("Compiler.cflags attribute must be str.")
        self._cflags = value

    @property
    def cfile(self):
        return self._cfile

    @cfile.setter
    def cfile(self, value):
        if value is not None:
            raise ValueError(
                "custom kernel files are not supported by the GPU library")
        self._cfile = value

    def compile(self, dimension, density, float_precision, operator):
        """Path of the shared object exporting ``forward`` for this variant.

        Same arguments as compiler.py:115-134: ``density`` is
        ``'constant_density'`` or ``'variable_density'``, ``float_precision``
        ``'-DFLOAT'`` or ``'-DDOUBLE'``; only ``operator='forward'`` exists.
        """
        if operator != 'forward':
            raise ValueError("Only forward operator available.")
        if dimension not in (2, 3):
            raise ValueError("dimension must be 2 or 3")
        if density not in ('constant_density', 'variable_density'):
            raise ValueError("unknown density variant " + str(density))
        if float_precision not in ('-DFLOAT', '-DDOUBLE'):
            raise ValueError("unknown precision " + str(float_precision))
        _lib.ensure_built()
        return _lib.shim_path(dimension, density == 'variable_density',
                              float_precision == '-DDOUBLE')
