"""The prebuilt large-scale optical tables of optical_elements.py:964-2120.

Each reference table is a grid of lossy beam splitters (``BS_symmetric``)
whose outputs travel right (port c) and down (port d) to the next splitters,
with free-space propagation or a building block on each edge, and
objective-lens detectors at the grid's edges.  Here every table is written as
data -- its sources, splitter angles, edges and detectors -- and one grid
executor runs it:

* splitter (i, j) takes ``a`` from above (a top source in row 0, else the d
  port of splitter (i-1, j) through the vertical edge) and ``b`` from the
  left (a left source in column 0, else the c port of (i, j-1) through the
  horizontal edge); with one input absent it is ``BS_symmetric_SI`` on the
  matching port (port 0 for ``a``, port 1 for ``b``);
* an edge is ``None`` (the light passes unchanged), a VRS over a distance, or
  a building block (sSLM [with amplitude] -> VRS -> LCD) followed by a VRS;
* a detector is ``VCZT_objective_lens`` of a splitter port, optionally after a
  VRS.

Distances, angles and mask settings follow the reference's parametrisation
(``(|p| * 100 + offset) cm`` and ``p * 2 pi - pi``) and may be tensors that
require grad: the gradients of splitter angles, distances, LCD settings and
phase masks all run through the hand-written adjoints.
"""
from __future__ import annotations

import numpy as np
import torch

from . import cm, engine

# ------------------------------------------------------------ parameters --


def _abs(p):
    return torch.abs(p) if isinstance(p, torch.Tensor) else np.abs(p)


def _angle(p):
    """optical_elements.py:1041-1056 etc.: a raw parameter in (0, 1) to (-pi, pi)."""
    return p * 2 * np.pi - np.pi


def _dist(p, offset):
    """optical_elements.py:1039-1040 etc.: (|p| * 100 + offset) cm, in float64
    (a float32 distance of 10 cm is off by ~0.01 um, a tenth of a radian of
    phase at visible wavelengths)."""
    if isinstance(p, torch.Tensor):
        p = p.to(torch.float64)
    return (_abs(p) * 100 + offset) * cm


# ----------------------------------------------------------------- edges --

def vrs(z):
    """Edge: free-space VRS over ``z``."""
    return ("vrs", z)


def block(alpha, phi, z1, eta, theta, z2):
    """Edge: building_block (sSLM -> VRS(z1) -> LCD) then VRS(z2), optical_elements.py:919-939."""
    return ("bb", alpha, phi, z1, eta, theta, z2)


def block_amp(alpha, phi, a1, a2, z1, eta, theta, z2):
    """Edge: bb_amplitude_and_phase_mod then VRS(z2), optical_elements.py:894-917."""
    return ("bba", alpha, phi, a1, a2, z1, eta, theta, z2)


def _run_edge(edge, light):
    from . import optical_elements as oe
    if edge is None:
        return light
    kind = edge[0]
    if kind == "vrs":
        return light.VRS_propagation(edge[1])[0]
    if kind == "bb":
        _, alpha, phi, z1, eta, theta, z2 = edge
        return oe.building_block(light, alpha, phi, z1, eta, theta).VRS_propagation(z2)[0]
    if kind == "bba":
        _, alpha, phi, a1, a2, z1, eta, theta, z2 = edge
        return oe.bb_amplitude_and_phase_mod(light, alpha, phi, a1, a2, z1, eta, theta).VRS_propagation(z2)[0]
    raise ValueError(f"unknown edge {kind!r}")


# -------------------------------------------------------------- executor --

def _splitter(a, b, theta):
    from . import optical_elements as oe
    if a is not None and b is not None:
        return oe.BS_symmetric(a, b, theta)
    if a is not None:
        return oe.BS_symmetric_SI(a, theta, port=0)
    if b is not None:
        return oe.BS_symmetric_SI(b, theta, port=1)
    raise ValueError("a splitter of the table has no input")


def _stack_lights(lights):
    """One light holding the (Ex, Ey) of lights on the same grid with no
    pending program, stacked along a new leading axis (flattened with the
    lights' own batch axes)."""
    from .vectorized_optics import VectorizedLight
    l0 = lights[0]
    ex = torch.stack([l.Ex for l in lights])
    ey = torch.stack([l.Ey for l in lights])
    ny, nx = ex.shape[-2:]
    return VectorizedLight._wrap(l0.x, l0.y, l0.wavelength, [ex.reshape(-1, ny, nx), ey.reshape(-1, ny, nx), None])


def _split_light(light, n, lead):
    """Undo _stack_lights: n lights of batch shape ``lead``."""
    from .vectorized_optics import VectorizedLight
    comps = [c.reshape((n,) + tuple(lead) + tuple(c.shape[-2:])) for c in (light.Ex, light.Ey, light.Ez)]
    return [VectorizedLight._wrap(light.x, light.y, light.wavelength, [c[k] for c in comps]) for k in range(n)]


def _z_per_field(z, lead):
    """A distance as a device float64 tensor with one value per field of a light of batch shape ``lead``."""
    from . import engine
    t = z if isinstance(z, torch.Tensor) else torch.full((), float(z), dtype=torch.float64, device=engine.device())
    t = t.to(dtype=torch.float64).reshape(-1) if t.numel() > 1 else t.to(dtype=torch.float64).reshape(())
    return t.expand(lead) if len(lead) else t.reshape(())


def _batchable(edge, light):
    return edge is not None and edge[0] == "vrs" and not light._ops


def _run_edges(jobs):
    """Run the edges leaving one wavefront of splitters.  Free-space edges of
    lights with no pending program and the same grid and wavelength run as
    one batched VRS with a distance per field; the others one by one."""
    out = [None] * len(jobs)
    groups = {}
    for k, (edge, light) in enumerate(jobs):
        if _batchable(edge, light):
            key = (engine.array_key(light.x), engine.array_key(light.y), float(light.wavelength),
                   tuple(light.Ex.shape))
            groups.setdefault(key, []).append(k)
        else:
            out[k] = _run_edge(edge, light)
    for ks in groups.values():
        if len(ks) == 1:
            out[ks[0]] = _run_edge(*jobs[ks[0]])
            continue
        lights = [jobs[k][1] for k in ks]
        lead = tuple(lights[0].Ex.shape[:-2])
        z = torch.stack([_z_per_field(jobs[k][0][1], lead) for k in ks]).reshape(-1)
        res, _ = _stack_lights(lights).VRS_propagation(z)
        for k, l in zip(ks, _split_light(res, len(ks), lead)):
            out[k] = l
    return out


def _detect(lights, r, f, xout, yout):
    """VCZT_objective_lens of every detector's light, as one batched focus
    where the lights allow it."""
    from . import optical_elements as oe
    l0 = lights[0]
    same = all(not l._ops and l.Ex.shape == l0.Ex.shape and l.wavelength == l0.wavelength and
               np.array_equal(l.x, l0.x) and np.array_equal(l.y, l0.y) for l in lights)
    if len(lights) < 2 or not same:
        return [oe.VCZT_objective_lens(l, r, f, xout, yout) for l in lights]
    det = oe.VCZT_objective_lens(_stack_lights(lights), r, f, xout, yout)
    return _split_light(det, len(lights), tuple(l0.Ex.shape[:-2]))


def _flatten_lights(lights):
    """(tensors, spec) of a list of lights (None kept as None): each light as
    its (Ex, Ey, Ez) planes, for a checkpointed segment's inputs / outputs."""
    flat, spec = [], []
    for light in lights:
        if light is None:
            spec.append(None)
            continue
        spec.append((light.x, light.y, light.wavelength))
        flat += [light.Ex, light.Ey, light.Ez]
    return flat, spec


def _unflatten_lights(flat, spec):
    from .vectorized_optics import VectorizedLight
    out, i = [], 0
    for sp in spec:
        if sp is None:
            out.append(None)
            continue
        out.append(VectorizedLight._wrap(sp[0], sp[1], sp[2], list(flat[i:i + 3])))
        i += 3
    return out


def run_grid(top, left, thetas, horizontal, vertical, detectors, r, f, xout, yout, checkpoint=False):
    """Run a splitter grid.

    top[j] / left[i]: source lights entering splitters (0, j) from above and
    (i, 0) from the left (None: no source); thetas[i][j]: splitter angles;
    horizontal[i][j]: the edge from (i, j)'s c port to (i, j+1);
    vertical[i][j]: the edge from (i, j)'s d port to (i+1, j); detectors: list
    of (i, j, port 'c' or 'd', edge).  Returns the detectors' lights.

    The grid runs by wavefronts (the splitters with i + j = k depend only on
    wavefront k - 1): the free-space edges leaving a wavefront run as one
    batched VRS, and the detectors as one batched focus.  ``checkpoint``
    (False, True, an int K or a checkpointing.CheckpointPolicy) stores only
    the inputs of every K-th wavefront, within a memory budget if the policy
    has one, and recomputes the others' fields in the backward."""
    from .checkpointing import CheckpointPolicy
    rows, cols = len(thetas), len(thetas[0])
    nwf = rows + cols - 1
    a_in = {(0, j): top[j] for j in range(cols)}
    b_in = {(i, 0): left[i] for i in range(rows)}
    det_in = [None] * len(detectors)

    def wavefront(k, a_in, b_in, det_in):
        cells = [(i, k - i) for i in range(rows) if 0 <= k - i < cols]
        jobs, targets = [], []
        for i, j in cells:
            c, d = _splitter(a_in.get((i, j)), b_in.get((i, j)), thetas[i][j])
            if j + 1 < cols:
                jobs.append((horizontal[i][j], c))
                targets.append(("b", (i, j + 1)))
            if i + 1 < rows:
                jobs.append((vertical[i][j], d))
                targets.append(("a", (i + 1, j)))
            for q, (di, dj, port, edge) in enumerate(detectors):
                if (di, dj) == (i, j):
                    jobs.append((edge, c if port == "c" else d))
                    targets.append(("det", q))
        for (kind, key), light in zip(targets, _run_edges(jobs)):
            if kind == "a":
                a_in[key] = light
            elif kind == "b":
                b_in[key] = light
            else:
                det_in[key] = light

    policy = CheckpointPolicy.coerce(checkpoint)
    if policy is None or not torch.is_grad_enabled():
        for k in range(nwf):
            wavefront(k, a_in, b_in, det_in)
        return _detect(det_in, r, f, xout, yout)

    from torch.utils.checkpoint import checkpoint as torch_checkpoint
    # output lights per wavefront, for the budget estimate
    n_out = [sum((j + 1 < cols) + (i + 1 < rows) + sum((di, dj) == (i, j) for di, dj, _, _ in detectors)
                 for i in range(rows) for j in [k - i] if 0 <= j < cols) for k in range(nwf)]
    src = next(l for l in list(top) + list(left) if l is not None)
    light_bytes = 3 * src.Ex.numel() * src.Ex.element_size()
    for k0, k1, ck in policy.segments(n_out, light_bytes):
        if not ck:
            for k in range(k0, k1):
                wavefront(k, a_in, b_in, det_in)
            continue
        # the segment's state: the lights entering wavefronts >= k0 and the detectors so far
        a_keys = sorted(key for key in a_in if sum(key) >= k0)
        b_keys = sorted(key for key in b_in if sum(key) >= k0)
        flat_in, spec_in = _flatten_lights([a_in[q] for q in a_keys] + [b_in[q] for q in b_keys] + det_in)
        out_spec = {}

        def seg(*flat, a_keys=a_keys, b_keys=b_keys, spec_in=spec_in, k0=k0, k1=k1, out_spec=out_spec):
            lights = _unflatten_lights(flat, spec_in)
            sa = dict(zip(a_keys, lights[:len(a_keys)]))
            sb = dict(zip(b_keys, lights[len(a_keys):len(a_keys) + len(b_keys)]))
            sd = list(lights[len(a_keys) + len(b_keys):])
            for k in range(k0, k1):
                wavefront(k, sa, sb, sd)
            ka = sorted(key for key in sa if sum(key) >= k1)
            kb = sorted(key for key in sb if sum(key) >= k1)
            fo, so = _flatten_lights([sa[q] for q in ka] + [sb[q] for q in kb] + sd)
            out_spec.update(ka=ka, kb=kb, spec=so)
            return tuple(fo)

        flat_out = torch_checkpoint(seg, *flat_in, use_reentrant=False)
        lights = _unflatten_lights(flat_out, out_spec["spec"])
        na, nb = len(out_spec["ka"]), len(out_spec["kb"])
        a_in = dict(zip(out_spec["ka"], lights[:na]))
        b_in = dict(zip(out_spec["kb"], lights[na:na + nb]))
        det_in = list(lights[na + nb:])
    return _detect(det_in, r, f, xout, yout)


def _ez_intensities(dets):
    return torch.stack([torch.abs(d.Ez) ** 2 for d in dets])


def _fluorescence_from(dets_ex, dets_dep):
    """optical_elements.py:1324-1345: normalised |Ex|^2 + |Ey|^2 of the
    excitation and depletion detectors, then the fluorescence model."""
    from . import optical_elements as oe

    def norm(d):
        i = torch.abs(d.Ex) ** 2 + torch.abs(d.Ey) ** 2
        return i / torch.sum(i)
    iex = torch.stack([norm(d) for d in dets_ex])
    idep = torch.stack([norm(d) for d in dets_dep])
    return oe.vectorized_fluorophores(iex, idep)


def _grid_3x3(thetas9):
    return [thetas9[0:3], thetas9[3:6], thetas9[6:9]]


_DETECTORS_3X3 = [(0, 2, "c"), (1, 2, "c"), (2, 2, "c"), (2, 0, "d"), (2, 1, "d"), (2, 2, "d")]


def _detectors(outs):
    return [(i, j, port, e) for (i, j, port), e in zip(_DETECTORS_3X3, list(outs) + [None] * 3)]


# ---------------------------------------------------------------- tables --

def _sharp_focus_edges(ph, eta, theta, z, z4, z5, block_edge):
    """The edges shared by robust_discovery, hybrid_setup_sharp_focus and
    hybrid_setup_fluorophores (optical_elements.py:1063-1094, 1595-1626,
    1742-1823): building blocks on (0,0)->(0,1), (1,1)->(1,2) and before
    detector 3; VRS(z4) / VRS(z5) down the middle and right columns."""
    (z11, z12), (z21, z22), (z31, z32) = z
    horizontal = [[block_edge(0, z11, z12), vrs(z21 + z22)],
                  [vrs(z11 + z12), block_edge(1, z21, z22)],
                  [vrs(z11 + z12), vrs(z21 + z22)]]
    vertical = [[None, vrs(z4), vrs(z4)],
                [None, vrs(z5), vrs(z5)]]
    outs = [vrs(z31 + z32), vrs(z31 + z32), block_edge(2, z31, z32)]
    return horizontal, vertical, outs


def _fixed_slms_edges(ph, eta, theta, z):
    """The edges of hybrid_setup_fixed_slms and its fluorophore variant
    (optical_elements.py:1449-1478, 1219-1307): fixed phase masks on
    (0,0)->(0,1), (1,1)->(1,2), (0,2)->(1,2) and (1,0)->(2,0)."""
    (z11, z12), (z21, z22), (z31, z32), (z41, z42) = z
    horizontal = [[block(ph[0][0], ph[0][1], z11, eta[0], theta[0], z12), vrs(z21 + z22)],
                  [vrs(z11 + z12), block(ph[1][0], ph[1][1], z21, eta[1], theta[1], z22)],
                  [vrs(z11 + z12), vrs(z21 + z22)]]
    vertical = [[None, vrs(z31 + z32), block(ph[2][0], ph[2][1], z31, eta[2], theta[2], z32)],
                [block(ph[3][0], ph[3][1], z41, eta[3], theta[3], z42), vrs(z41 + z42), vrs(z41 + z42)]]
    return horizontal, vertical, [None, None, None]


def _unpack_blocks(parameters, offset, n_blocks=3):
    """[phase_1, phase_2, eta, theta, z_1, z_2] per block (optical_elements.py:1553-1576)."""
    ph, eta, theta, z = [], [], [], []
    for b in range(n_blocks):
        p = parameters[6 * b:6 * b + 6]
        ph.append((_angle(p[0]), _angle(p[1])))
        eta.append(_angle(p[2]))
        theta.append(_angle(p[3]))
        z.append((_dist(p[4], offset), _dist(p[5], offset)))
    return ph, eta, theta, z


def robust_discovery(ls1, ls2, ls3, ls4, ls5, ls6, parameters, fixed_params, noise_distances, noise_slms,
                     noise_wps, noise_amps, distance_offset=15):
    """optical_elements.py:964-1117: the 3x3 table with amplitude-and-phase
    building blocks and noise on every setting; returns the detectors' |Ez|^2."""
    r, f, xout, yout = fixed_params[0:4]
    ph, amp, eta, theta, z = [], [], [], [], []
    for b in range(3):
        p = parameters[8 * b:8 * b + 8]
        ph.append((_angle(p[0]) + noise_slms[2 * b], _angle(p[1]) + noise_slms[2 * b + 1]))
        amp.append((p[2] + noise_amps[2 * b], p[3] + noise_amps[2 * b + 1]))
        eta.append(_angle(p[4]) + noise_wps[2 * b])
        theta.append(_angle(p[5]) + noise_wps[2 * b + 1])
        z.append((_dist(p[6], distance_offset) + noise_distances[2 * b],
                  _dist(p[7], distance_offset) + noise_distances[2 * b + 1]))
    thetas = [_angle(parameters[24 + k]) for k in range(9)]
    z4 = _dist(parameters[33], distance_offset) + noise_distances[6]
    z5 = _dist(parameters[34], distance_offset) + noise_distances[7]

    def blk(b, z1, z2):
        return block_amp(ph[b][0], ph[b][1], amp[b][0], amp[b][1], z1, eta[b], theta[b], z2)
    horizontal, vertical, outs = _sharp_focus_edges(ph, eta, theta, z, z4, z5, blk)
    dets = run_grid([ls1, ls2, ls3], [ls4, ls5, ls6], _grid_3x3(thetas), horizontal, vertical,
                    _detectors(outs), r, f, xout, yout)
    return _ez_intensities(dets)


def _table_batch(light, T):
    """A source light as a batch of T tables (stride-0 views, no copies)."""
    from .vectorized_optics import VectorizedLight
    ex, ey = light.Ex, light.Ey
    ny, nx = ex.shape[-2:]
    return VectorizedLight._wrap(light.x, light.y, light.wavelength,
                                 [ex.expand(T, ny, nx), ey.expand(T, ny, nx), None])


def batch_robust_discovery(ls1, ls2, ls3, ls4, ls5, ls6, parameters, fixed_params, noise_distances, noise_slms,
                           noise_wps, noise_amps, distance_offset=15):
    """robust_discovery over many noisy copies of one table
    (examples/noisy_optimization.ipynb, a vmap there): the noise arrays carry a
    leading table axis -- distances (T, 8), slms and amps (T, 6, R, R), wps
    (T, 6) -- and every table runs in the same launches, as one batch of T
    fields with per-table distances, masks and waveplate settings.  Returns
    the detected |Ez|^2 as (T, 6, M, M)."""
    T = noise_slms.shape[0]
    nd = noise_distances.reshape(T, -1)
    nw = noise_wps.reshape(T, -1)
    srcs = [_table_batch(ls, T) for ls in (ls1, ls2, ls3, ls4, ls5, ls6)]
    I = robust_discovery(*srcs, parameters, fixed_params, [nd[:, k] for k in range(nd.shape[1])],
                         [noise_slms[:, k] for k in range(noise_slms.shape[1])], [nw[:, k] for k in range(nw.shape[1])],
                         [noise_amps[:, k] for k in range(noise_amps.shape[1])], distance_offset)
    return I.transpose(0, 1)


def hybrid_setup_sharp_focus(ls1, ls2, ls3, ls4, ls5, ls6, parameters, fixed_params, distance_offset=8.9,
                             checkpoint=False):
    """optical_elements.py:1503-1649: returns (stacked |Ez|^2 of the six
    detectors, the detectors' lights).  ``checkpoint``: see run_grid."""
    r, f, xout, yout = fixed_params[0:4]
    ph, eta, theta, z = _unpack_blocks(parameters, distance_offset)
    thetas = [_angle(parameters[18 + k]) for k in range(9)]
    z4, z5 = _dist(parameters[27], distance_offset), _dist(parameters[28], distance_offset)

    def blk(b, z1, z2):
        return block(ph[b][0], ph[b][1], z1, eta[b], theta[b], z2)
    horizontal, vertical, outs = _sharp_focus_edges(ph, eta, theta, z, z4, z5, blk)
    dets = run_grid([ls1, ls2, ls3], [ls4, ls5, ls6], _grid_3x3(thetas), horizontal, vertical,
                    _detectors(outs), r, f, xout, yout, checkpoint=checkpoint)
    return _ez_intensities(dets), dets


def hybrid_setup_fluorophores(ls1, ls2, ls3, ls4, ls5, ls6, parameters, fixed_params, distance_offset=8.9):
    """optical_elements.py:1651-1853: the sharp-focus table run twice, the
    depletion beam (ls1, ls3, ls5) and the excitation beam (ls2, ls4, ls6)
    entering different ports; returns the fluorescence of the six detectors."""
    r, f, xout, yout = fixed_params[0:4]
    ph, eta, theta, z = _unpack_blocks(parameters, distance_offset)
    thetas = _grid_3x3([_angle(parameters[18 + k]) for k in range(9)])
    z4, z5 = _dist(parameters[27], distance_offset), _dist(parameters[28], distance_offset)

    def blk(b, z1, z2):
        return block(ph[b][0], ph[b][1], z1, eta[b], theta[b], z2)
    horizontal, vertical, outs = _sharp_focus_edges(ph, eta, theta, z, z4, z5, blk)
    dets_r = run_grid([ls1, None, ls3], [None, ls5, None], thetas, horizontal, vertical, _detectors(outs),
                      r, f, xout, yout)
    dets_g = run_grid([None, ls2, None], [ls4, None, ls6], thetas, horizontal, vertical, _detectors(outs),
                      r, f, xout, yout)
    return _fluorescence_from(dets_g, dets_r)


def _fixed_slms_params(parameters, fixed_params, offset):
    ph = [(fixed_params[4], fixed_params[5]), (fixed_params[6], fixed_params[6]),
          (fixed_params[7], fixed_params[7]), (fixed_params[8], fixed_params[9])]
    z = [(_dist(parameters[2 * b], offset), _dist(parameters[2 * b + 1], offset)) for b in range(4)]
    thetas = _grid_3x3([_angle(parameters[8 + k]) for k in range(9)])
    eta = [_angle(parameters[17 + 2 * b]) for b in range(4)]
    theta = [_angle(parameters[18 + 2 * b]) for b in range(4)]
    return ph, z, thetas, eta, theta


def hybrid_setup_fixed_slms(ls1, ls2, ls3, ls4, ls5, ls6, parameters, fixed_params, distance_offset=8.9):
    """optical_elements.py:1347-1501: fixed phase masks (fixed_params[4:10]) at
    four places of the 3x3 table; returns (stacked |Ez|^2, detectors)."""
    r, f, xout, yout = fixed_params[0:4]
    ph, z, thetas, eta, theta = _fixed_slms_params(parameters, fixed_params, distance_offset)
    horizontal, vertical, outs = _fixed_slms_edges(ph, eta, theta, z)
    dets = run_grid([ls1, ls2, ls3], [ls4, ls5, ls6], thetas, horizontal, vertical, _detectors(outs),
                    r, f, xout, yout)
    return _ez_intensities(dets), dets


def hybrid_setup_fixed_slms_fluorophores(ls1, ls2, ls3, ls4, ls5, ls6, parameters, fixed_params,
                                         distance_offset=8.9):
    """optical_elements.py:1119-1345: the fixed-mask table for the depletion
    (ls1, ls3, ls5) and excitation (ls2, ls4, ls6) beams; returns the
    fluorescence of the six detectors."""
    r, f, xout, yout = fixed_params[0:4]
    ph, z, thetas, eta, theta = _fixed_slms_params(parameters, fixed_params, distance_offset)
    horizontal, vertical, outs = _fixed_slms_edges(ph, eta, theta, z)
    dets_r = run_grid([ls1, None, ls3], [None, ls5, None], thetas, horizontal, vertical, _detectors(outs),
                      r, f, xout, yout)
    dets_g = run_grid([None, ls2, None], [ls4, None, ls6], thetas, horizontal, vertical, _detectors(outs),
                      r, f, xout, yout)
    return _fluorescence_from(dets_g, dets_r)


def six_times_six_ansatz(ls1, ls2, ls3, ls4, ls5, ls6, ls7, ls8, ls9, ls10, ls11, ls12, parameters, fixed_params,
                         distance_offset=7.6):
    """optical_elements.py:1855-2120: a 6x6 splitter grid with two fixed-mask
    building blocks; returns the |Ez|^2 of its twelve detectors (the right
    column's c ports, the bottom row's c ports of columns 0-4 -- which also
    travel on to the right, as in the reference -- and the last d port)."""
    r, f, xout, yout = fixed_params[0:4]
    (p11, p12, p21, p22) = fixed_params[4:8]
    z = [_dist(parameters[k], distance_offset) for k in range(12)]
    bs = [_angle(parameters[12 + k]) for k in range(36)]
    eta1, theta1, eta2, theta2 = (_angle(parameters[48 + k]) for k in range(4))
    thetas = [bs[6 * i:6 * i + 6] for i in range(6)]
    row = [vrs(z[0]), vrs(z[1] + z[2]), vrs(z[3]), vrs(z[4] + z[5]), vrs(z[6])]
    horizontal = [list(row) for _ in range(6)]
    horizontal[1][1] = block(p11, p12, z[1], eta1, theta1, z[2])
    horizontal[3][3] = block(p21, p22, z[4], eta2, theta2, z[5])
    vertical = [[vrs(z[7 + i])] * 6 for i in range(5)]
    detectors = [(i, 5, "c", None) for i in range(6)] + [(5, j, "c", None) for j in range(5)] + [(5, 5, "d", None)]
    dets = run_grid([ls1, ls2, ls3, ls4, ls5, ls6], [ls7, ls8, ls9, ls10, ls11, ls12], thetas, horizontal,
                    vertical, detectors, r, f, xout, yout)
    return _ez_intensities(dets)
