"""Gradients of radargram power: a hand-written adjoint behind
``torch.autograd.Function``.

The reference has no gradient code; this module adds one for the refracted
target path of ``kernels/multilayer.py:594-770`` (coherent mode; the
sequential chain or the joint solve of ``refraction_joint.py:249-322``).
``WindowPowerModel`` fixes the scene, track and instrument;
its differentiable map

    (reflectivity_db (N,), rms_height (N,), alpha) -> P (T,)

gives each trace's power summed over a fast-time window of the target's
field, P_t = sum_{b in window} |F_t[b]|^2, with

* reflectivity_db: per-facet reflection coefficient in dB, gamma = 10^(R/20);
* rms_height: per-facet roughness rms height sigma (the rough-facet model
  of ``kernels/coherent.py:131-168``, series of ``roughness.py:127-186``);
* alpha: attenuation rate (dB/km) of the legs listed in ``alpha_legs``
  (indices into the caller's ``att_leg``).

Forward: ``ss_refracted_fwd`` (split form, or the FP64 form). Backward:
``ss_refracted_adjoint`` recomputes every (trace, facet) phasor from the
geometry -- nothing per pair is stored -- with a fix-up pass for the few
pairs that need float64 lookup or bin decisions, and returns dL/dR,
dL/dsigma and dL/dalpha for the upstream dL/dP. Any loss built from P with torch operations (e.g. the squared dB
misfit of ``db_misfit``) then differentiates end to end.
"""

import ctypes as C

import numpy as np
import torch

from . import _lib
from .multilayer import prepare_refracted


class WindowPowerModel:
    """Scene, track and instrument of a differentiable bed-power map."""

    def __init__(self, positions, u_ct, target, crossed, eps_leg, att_leg, *,
                 t0, dt, n_samples, c, k0, window, alpha_legs,
                 corr_length, phasors, n_terms, acf="exponential",
                 d_phi_area=True, taper_s=0.05, refraction="sequential",
                 pad_to=None, joint_newton=6, joint_backtrack=4,
                 precision="split", device=None):
        n = np.asarray(target.centers).shape[0]
        self.N = n
        self.window = (int(window[0]), int(window[1]))
        self.alpha_legs = tuple(int(v) for v in alpha_legs)
        self.plan = prepare_refracted(
            positions, u_ct, target, crossed, eps_leg, att_leg,
            mode="coherent", t0=t0, dt=dt, n_samples=n_samples, c=c,
            gamma=np.ones(n), k0=k0,
            roughness=(np.full(n, 0.1), corr_length, phasors, n_terms, acf),
            d_phi_area=d_phi_area, taper_s=taper_s, refraction=refraction,
            pad_to=pad_to, joint_newton=joint_newton,
            joint_backtrack=joint_backtrack, precision=precision,
            device=device)
        self.device = self.plan.device
        self.order = torch.as_tensor(self.plan.cull.order, device=self.device)
        # the joint solve pads air planes (and legs) above the surface
        self.k_pad = int(self.plan.opts.k_pad) if refraction == "joint" else 0
        mask = np.zeros(len(self.plan.legs[2]))
        for leg in self.alpha_legs:
            mask[leg + self.k_pad] = 1.0
        self.alpha_mask = np.ascontiguousarray(mask, np.float64)
        self.scratch = None
        lo, hi = self.window
        if not 0 <= lo < hi <= self.plan.n_seg:
            raise ValueError("window outside [0, n_samples)")

    # -- parameter upload (facet arrays are in the plan's along-track order)
    def _set(self, reflectivity_db, rms_height, alpha):
        ex = self.plan.fac.extras
        R = reflectivity_db.detach().to(self.device, torch.float64)
        ex["gamma_f64"].copy_(torch.pow(10.0, R[self.order] / 20.0))
        s = rms_height.detach().to(self.device, torch.float32)
        ex["sigma"].copy_(s[self.order])
        a = float(alpha)
        for leg in self.alpha_legs:
            self.plan.legs[2][leg + self.k_pad] = a

    def forward_field(self, reflectivity_db, rms_height, alpha):
        """Target field (T, n_samples, 2) float64 for these parameters."""
        self._set(reflectivity_db, rms_height, alpha)
        field, _ = self.plan.run()
        return field

    def window_power(self, field):
        lo, hi = self.window
        return (field[:, lo:hi, :] ** 2).sum(dim=(1, 2))

    def adjoint(self, field, grad_power):
        """dL/dR (N,), dL/dsigma (N,) and dL/dalpha for upstream dL/dP."""
        L = _lib.lib()
        N = self.N
        blocks = L.ss_refracted_adjoint_blocks(N)
        gR = torch.empty(N, dtype=torch.float64, device=self.device)
        gS = torch.empty(N, dtype=torch.float64, device=self.device)
        gA = torch.empty(blocks, dtype=torch.float64, device=self.device)
        gP = grad_power.detach().to(self.device, torch.float64).contiguous()
        field = field.contiguous()
        nbytes = L.ss_refracted_adjoint_scratch_bytes(self.plan.T, N)
        if self.scratch is None or self.scratch.numel() < nbytes:
            self.scratch = torch.empty(nbytes, dtype=torch.uint8,
                                       device=self.device)
        io = _lib.AdjointIO(field.data_ptr(), gP.data_ptr(), self.window[0],
                            self.window[1],
                            self.alpha_mask.ctypes.data_as(C.c_void_p),
                            gR.data_ptr(), gS.data_ptr(), gA.data_ptr(),
                            self.scratch.data_ptr(), nbytes)
        p = self.plan
        stream = torch.cuda.current_stream(self.device).cuda_stream
        st = L.ss_refracted_adjoint(C.byref(p.opts), C.byref(p.fst),
                                    C.byref(p.tr), C.byref(p.pst),
                                    C.byref(p.rst), C.byref(io),
                                    C.c_void_p(stream))
        _lib.check(st, "ss_refracted_adjoint")
        # back to the caller's facet order
        outR = torch.empty_like(gR)
        outS = torch.empty_like(gS)
        outR[self.order] = gR
        outS[self.order] = gS
        return outR, outS, gA.sum()

    def power(self, reflectivity_db, rms_height, alpha):
        """Differentiable P (T,) for these parameters."""
        return WindowPower.apply(reflectivity_db, rms_height, alpha, self)


class WindowPower(torch.autograd.Function):
    """P_t = sum_{b in window} |F_t[b]|^2 with a hand-written backward."""

    @staticmethod
    def forward(ctx, reflectivity_db, rms_height, alpha, model):
        field = model.forward_field(reflectivity_db, rms_height, alpha)
        ctx.model = model
        ctx.save_for_backward(field, reflectivity_db.detach().clone(),
                              rms_height.detach().clone(),
                              torch.as_tensor(alpha).detach().clone())
        return model.window_power(field)

    @staticmethod
    def backward(ctx, grad_power):
        field, R, s, a = ctx.saved_tensors
        model = ctx.model
        model._set(R, s, a)  # the adjoint reads the forward's parameters
        gR, gS, gA = model.adjoint(field, grad_power)
        return (gR.to(device=R.device, dtype=R.dtype),
                gS.to(device=s.device, dtype=s.dtype),
                gA.to(device=a.device, dtype=a.dtype), None)


def db_misfit(P, P_target):
    """L = sum_t (10 log10 P_t - 10 log10 Phat_t)^2 (the bed-echo power
    misfit of the differentiation configuration)."""
    return ((10.0 * torch.log10(P) - 10.0 * torch.log10(P_target)) ** 2).sum()
