"""Restatement of the inversion drivers' model-update arithmetic in numpy.

TEST INFRASTRUCTURE ONLY: tests/ compare the host library's update routines
(sfwi_gb300/host/sfwi_host.cpp, used by the sfwi_fwi driver) with this file,
bit for bit.  Nothing in the product imports it.

It follows the reference line by line, with its operand types:
  - every array element is a float32, every product or quotient of two of
    them a float32 (numpy float32 arithmetic rounds each operation to single
    precision and never fuses a multiply into an add);
  - the CG scalars (beta_fenzi, beta_fenmu, beta, alpha, fenzi, fenmu) are
    doubles; a double times a float32 element is formed in double and the
    result stored back as float32;
  - beta_fenzi is a sequential double sum over the cells in i-major order.
Stage 1: sfwi-stage1/main.cpp:35-49 (normalize_all), :64-73 (cal_step2),
:687-750 (preconditioning, cut layer, CG), :832-841 (line-search direction),
:1222-1237 (step and clamp), :1247-1264 (update, cut-layer flattening).
Stage 2: sfwi-stage2/main.cpp:646-703 (cut, preconditioning, CG) and
:865-875 (alpha = fenzi/fenmu, image update).
"""
import numpy as np

F32, F64 = np.float32, np.float64
CUT_LAYER = 26  # cut_layer, sfwi-stage1/main.cpp:410; the literal 26 in sfwi-stage2/main.cpp:648


def _seq_sum(terms):
    """0.0 + t[0] + t[1] + ... in double, left to right (the reference's
    `beta_fenzi += ...` inside its i, j loops)"""
    t = np.asarray(terms, F64).ravel()
    return float(np.add.accumulate(t)[-1]) if t.size else 0.0


def normalize_all(a, b):
    """sfwi-stage1/main.cpp:35-49: both divided by the largest |value| of the two"""
    m = F32(max(np.abs(a).max(), np.abs(b).max()))
    return (a / m).astype(F32), (b / m).astype(F32)


class State:
    """pp_cg_old, ps_cg_old and beta_fenmu across iterations"""

    def __init__(self, shape):
        self.old_pp = np.zeros(shape, F32)
        self.old_ps = np.zeros(shape, F32)
        self.beta_fenmu = 0.0


def _recurrence(st, beta, cp, cs):
    # main.cpp:739-748: pp_cg = pp_cg + beta * pp_cg_old (double), then the copy
    cp = (cp.astype(F64) + beta * st.old_pp.astype(F64)).astype(F32)
    cs = (cs.astype(F64) + beta * st.old_ps.astype(F64)).astype(F32)
    st.old_pp, st.old_ps = cp.copy(), cs.copy()
    return cp, cs


def stage1_direction(st, it, grad_pp, grad_ps, illum):
    """(beta, cg_pp, cg_ps, d_pp, d_ps)"""
    grad_pp, grad_ps, illum = (np.asarray(a, F32) for a in (grad_pp, grad_ps, illum))
    with np.errstate(divide="ignore", invalid="ignore"):
        sp = (grad_pp / illum).astype(F32)        # main.cpp:696-697
        ss = (grad_ps / illum).astype(F32)
    sp[:, :CUT_LAYER] = 0.0                        # :706-709
    ss[:, :CUT_LAYER] = 0.0
    beta_fenzi = _seq_sum(grad_pp * sp + grad_ps * ss)   # :723 (float terms)
    beta = 0.0 if it == 0 else beta_fenzi / st.beta_fenmu  # :729-735
    cp, cs = _recurrence(st, beta, sp, ss)
    st.beta_fenmu = beta_fenzi                     # :750
    d_pp, d_ps = normalize_all(cp, cs)             # :832-841
    return beta, cp, cs, d_pp, d_ps


def stage1_alpha(m0, m1, m2, step1=30.0, step2=150.0):
    """cal_step2 (main.cpp:64-73) and the clamp (:1230-1237)"""
    s1, s2 = F32(step1), F32(step2)
    fenzi = float(s1 * s1 - s2 * s2) * m0 + float(s2 * s2) * m1 + float(-s1 * s1) * m2
    fenmu = float(s1 - s2) * m0 + float(s2) * m1 + float(-s1) * m2
    alpha = fenzi / fenmu / 2.0
    if alpha > 300:
        alpha = 300.0
    if alpha < -100:
        alpha = -100.0
    return alpha


def stage1_update(alpha, d_pp, d_ps, vp, vs):
    """main.cpp:1247-1264; returns the new (vp, vs)"""
    vp = (np.asarray(vp, F32).astype(F64) - alpha * np.asarray(d_pp, F32).astype(F64)).astype(F32)
    vs = (np.asarray(vs, F32).astype(F64) - alpha * np.asarray(d_ps, F32).astype(F64)).astype(F32)
    vp[:, :CUT_LAYER] = vp[0, 0]
    vs[:, :CUT_LAYER] = vs[0, 0]
    return vp, vs


def stage2_direction(st, it, grad_pp, grad_ps, illum):
    """(beta, grad_pp, grad_ps, cg_pp, cg_ps) with the gradients zeroed above the cut"""
    gp, gs = (np.array(a, F32) for a in (grad_pp, grad_ps))
    illum = np.asarray(illum, F32)
    gp[:, :CUT_LAYER] = 0.0                        # sfwi-stage2/main.cpp:663-664
    gs[:, :CUT_LAYER] = 0.0
    with np.errstate(divide="ignore", invalid="ignore"):
        cp = (gp / illum).astype(F32)              # :656-657
        cs = (gs / illum).astype(F32)
        cp[:, :CUT_LAYER] = 0.0                    # :665-666
        cs[:, :CUT_LAYER] = 0.0
        beta_fenzi = _seq_sum(gp * gp / illum + gs * gs / illum)  # :670
    beta = 0.0 if it == 0 else beta_fenzi / st.beta_fenmu     # :674-679
    cp, cs = _recurrence(st, beta, cp, cs)         # :692-701
    st.beta_fenmu = beta_fenzi                     # :703
    return beta, gp, gs, cp, cs


def stage2_update(fenzi, fenmu, cg_pp, cg_ps, image_pp, image_ps):
    """sfwi-stage2/main.cpp:865-875; returns (alpha, image_pp, image_ps)"""
    alpha = fenzi / fenmu
    ip = (np.asarray(image_pp, F32).astype(F64) - alpha * np.asarray(cg_pp, F32).astype(F64)).astype(F32)
    ips = (np.asarray(image_ps, F32).astype(F64) - alpha * np.asarray(cg_ps, F32).astype(F64)).astype(F32)
    return alpha, ip, ips
