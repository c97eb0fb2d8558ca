"""Unit conversions between physical units and simulation units (cardiax/convert.py:1-67).

Pure host arithmetic; same truncation semantics as the reference (``int(x / step)``).
"""


def params_to_units(params, dx, dt):
    """Rescale a dict of parameters to simulation units (cardiax/convert.py:5-16)."""
    params = dict(params)
    params["Cm"] /= (dx ** 2) / dt
    for k in ("tau_d", "tau_v1_minus", "tau_v2_minus", "tau_v_plus", "tau_0", "tau_r",
              "tau_si", "tau_w_minus", "tau_w_plus"):
        params[k] /= dt
    return params


def diffusivity_to_units(d, dt):
    return d / dt


def diffusivity_rescale(c, domain):
    """Affine map of ``c`` onto [domain[0], domain[1]] (cardiax/convert.py:24-27)."""
    a, b = c.min(), c.max()
    y, z = domain[0], domain[1]
    return (c - a) * (z - y) / (b - a) + y


def realsize_to_shape(field, dx):
    return (int(field[0] / dx), int(field[1] / dx))


def shape_to_realsize(field, dx):
    return (int(field[0] * dx), int(field[1] * dx))


def cm_to_units(value, dx):
    return int(value / dx)


def units_to_cm(value, dx):
    return value * dx


def ms_to_units(value, dt):
    return int(value / dt)


def units_to_ms(value, dt):
    return value * dt


def stimuli_to_units(stimuli, dx, dt):
    """``start``, ``duration`` and ``period`` of each stimulus mapping converted from ms to
    steps, in place (cardiax/convert.py:53-59)."""
    stimuli = list(stimuli)
    for s in stimuli:
        for key in ("start", "duration", "period"):
            s[key] = ms_to_units(s[key], dt)
    return stimuli


def u_to_V(u, V0=-85, Vfi=15):
    return ((Vfi - V0) * u) + V0


def V_to_u(V, V0=-85, Vfi=15):
    return (V - V0) / (Vfi - V0)
