"""The example-stax layer factories the reference builds on, restated from their documented
behaviour: each returns (init_fn(rng, input_shape) -> (output_shape, params),
apply_fn(params, inputs, **kw)). Only shapes and forward values are provided."""
import numpy as np

from .. import lax, random
from .._missing import missing_attr


def GeneralConv(dimension_numbers, out_chan, filter_shape, strides=None,  # noqa: N802
                padding='VALID', W_init=None, b_init=None):
    lhs_spec, rhs_spec, out_spec = dimension_numbers
    strides = tuple(strides or (1,) * len(filter_shape))
    draw_w = W_init or random.normal
    draw_b = b_init or random.normal

    def weight_shape(input_shape):
        it = iter(filter_shape)
        return [out_chan if c == 'O' else input_shape[lhs_spec.index('C')] if c == 'I'
                else next(it) for c in rhs_spec]

    def init_fn(rng, input_shape):
        ws = weight_shape(input_shape)
        out_shape = lax.conv_general_shape_tuple(input_shape, ws, strides, padding,
                                                 dimension_numbers)
        bs = [out_chan if c == 'C' else 1 for c in out_spec]
        k1, k2 = random.split(rng)
        return out_shape, (draw_w(k1, ws), draw_b(k2, bs))

    def apply_fn(params, inputs, **_):
        w, b = params
        return lax.conv_general_dilated(inputs, w, strides, padding,
                                        dimension_numbers=dimension_numbers) + b

    return init_fn, apply_fn


def _window_layer(average):
    def make(window_shape, strides=None, padding='VALID', spec=None):
        strides = tuple(strides or (1,) * len(window_shape))
        nd = len(window_shape) + 2
        n_ax, c_ax = (0, nd - 1) if spec is None else (spec.index('N'), spec.index('C'))
        win, st = [], []
        it_w, it_s = iter(window_shape), iter(strides)
        for a in range(nd):
            if a in (n_ax, c_ax):
                win.append(1)
                st.append(1)
            else:
                win.append(next(it_w))
                st.append(next(it_s))

        def init_fn(rng, input_shape):
            return lax.reduce_window_shape_tuple(input_shape, win, st, padding), ()

        def apply_fn(params, inputs, **_):
            total = lax.reduce_window(inputs, 0., lax.add, win, st, padding)
            if not average:
                return total
            # the mean over the window's entries that lie inside the input
            ones = np.ones([1 if a in (n_ax, c_ax) else np.shape(inputs)[a] for a in range(nd)])
            count = lax.reduce_window(ones, 0., lax.add, win, st, padding)
            return total / count

        return init_fn, apply_fn
    return make


AvgPool = _window_layer(True)
SumPool = _window_layer(False)


def _identity():
    return (lambda rng, input_shape: (input_shape, ())), (lambda params, inputs, **_: inputs)


Identity = _identity()  # a layer pair, not a factory


def serial(*layers):
    inits, applies = zip(*layers) if layers else ((), ())

    def init_fn(rng, input_shape):
        params = []
        for f in inits:
            rng, sub = random.split(rng)
            input_shape, p = f(sub, input_shape)
            params.append(p)
        return input_shape, params

    def apply_fn(params, inputs, **kw):
        for f, p in zip(applies, params):
            inputs = f(p, inputs, **kw)
        return inputs

    return init_fn, apply_fn


def parallel(*layers):
    inits, applies = zip(*layers) if layers else ((), ())

    def init_fn(rng, input_shape):
        keys = random.split(rng, len(inits))
        res = [f(k, s) for f, k, s in zip(inits, keys, input_shape)]
        return [r[0] for r in res], [r[1] for r in res]

    def apply_fn(params, inputs, **kw):
        return [f(p, x, **kw) for f, p, x in zip(applies, params, inputs)]

    return init_fn, apply_fn


def softmax(x, axis=-1):
    e = np.exp(x - np.max(x, axis=axis, keepdims=True))
    return e / np.sum(e, axis=axis, keepdims=True)


def __getattr__(name):
    return missing_attr('example_libraries.stax.' + name, placeholder=True)
