"""Learned surrogate of the species rates, with per-state fallback to FP64.

Network: MLP 54 -> 4 x 256 SiLU -> 53 (+1), BF16 weights and activations,
FP32 accumulation, every layer a hand-written tcgen05 GEMM (mlp_ops /
csrc/pjg_mlp.cu) for inference and for training (forward, input gradients,
weight gradients).  Inputs are log-scaled states: (T, ln P, log10 c_k for the
52 non-bath species).  Outputs are the 53 rates {dT/dt, dn_0/dt .. dn_51/dt}
(the extra-variable rate is recomputed from them exactly as the FP64 path does,
rate_subs.py get_extra_var_rates :798-960), each mapped through
asinh(y / s_k) and standardised.  The 54th output estimates log10 of the
state's relative error; states whose estimate exceeds the tolerance (or whose
inputs leave the training box) are evaluated by the FP64 kernel instead.

Training loss (Sobolev): mean squared error of the standardised outputs plus
mean squared error of directional derivatives along random input directions
u, where the network derivative is a central difference of the network and
the target J u comes from the FP64 analytical Jacobian kernel (pjg_jacobian).
The FP64 path stays the reference and the fallback.
"""
import math
import os
import time

import numpy as np
import torch

from . import _lib, api, mlp_ops
from .mech.elements import RU

HID = 256
NIN, NIN_P = 54, 64
NOUT, NOUT_P = 53, 64
ERR = NOUT          # output column of the error estimate
FEAT_FLOOR = 1e-20  # concentration floor of the log features


class MLP(object):
    """Weights (FP32 master + BF16 copies) and the tcgen05 forward/backward.
    depth: hidden layers of width HID (4 for the product network; the fused
    single-launch inference is built for 4)."""

    def __init__(self, device, seed=0, depth=4):
        self.device = device
        self.depth = int(depth)
        self.dims = [(NIN_P, HID)] + [(HID, HID)] * (self.depth - 1) + [(HID, NOUT_P)]
        g = torch.Generator().manual_seed(seed)
        self.W, self.b = [], []
        for din, dout in self.dims:
            w = torch.randn(dout, din, generator=g, dtype=torch.float64) * math.sqrt(1.7 / din)
            self.W.append(w.float().to(device))
            self.b.append(torch.zeros(dout, device=device))
        self.W[0][:, NIN:] = 0.0
        self.W[-1][ERR + 1:, :] = 0.0
        self.W[-1] *= 0.3
        self.mask_in = torch.zeros(HID, NIN_P, device=device)
        self.mask_in[:, :NIN] = 1.0
        self.mask_out = torch.zeros(NOUT_P, HID, device=device)
        self.mask_out[:ERR + 1] = 1.0
        self.m = [torch.zeros_like(w) for w in self.W] + [torch.zeros_like(b) for b in self.b]
        self.v = [torch.zeros_like(w) for w in self.W] + [torch.zeros_like(b) for b in self.b]
        self.t = 0
        self._buf = {}
        self.refresh()

    def refresh(self):
        self.Wb = [w.to(torch.bfloat16).contiguous() for w in self.W]
        self.Wtb = [w.t().contiguous().to(torch.bfloat16) for w in self.W]
        # operands of the fused forward (4 hidden layers only)
        self.Wp = [mlp_ops.pack_core(w) for w in self.Wb] if self.depth == 4 else None

    def _get(self, key, shape, dtype):
        b = self._buf.get(key)
        if b is None or b.shape != shape or b.dtype != dtype:
            b = torch.empty(shape, dtype=dtype, device=self.device)
            self._buf[key] = b
        return b

    def forward(self, X, keep=False, out=None):
        """X: [M, 64] BF16 -> [M, 64] FP32.  keep=True stores what backward needs."""
        M = X.shape[0]
        a = X
        self.saved = [] if keep else None
        for l in range(self.depth):
            A = self._get(("A", l, keep), (M, HID), torch.bfloat16)
            Z = self._get(("Z", l), (M, HID), torch.bfloat16) if keep else None
            AT = self._get(("AT", l), (HID, M), torch.bfloat16) if keep else None
            mlp_ops.linear(a, self.Wb[l], bias=self.b[l], act=True, Y=A, YT=AT, Z=Z)
            if keep:
                self.saved.append((Z, AT))
            a = A
        Y = out if out is not None else self._get(("Y", keep), (M, NOUT_P), torch.float32)
        mlp_ops.linear(a, self.Wb[-1], bias=self.b[-1], Y32=Y)
        return Y

    def infer(self, X, out=None):
        """Inference: the whole network in one fused tcgen05 launch (activations
        stay on chip); same result as forward(X).  Other depths run layer by
        layer."""
        if self.Wp is None:
            return self.forward(X, out=out)
        return mlp_ops.forward_fused(X, self.Wp, self.b, Y=out)

    def backward(self, XT, dY):
        """Weight and bias gradients for the last forward(keep=True); XT = X^T [64, M]."""
        M = dY.shape[0]
        gW = [torch.zeros_like(w) for w in self.W]
        gb = [torch.zeros_like(b) for b in self.b]
        L = self.depth
        gb[L] = dY.sum(0)
        dZ = dY.to(torch.bfloat16).contiguous()
        dZT = dZ.t().contiguous()
        for l in range(L, -1, -1):
            inT = XT if l == 0 else self.saved[l - 1][1]
            mlp_ops.wgrad(dZT, inT, gW[l])
            if l > 0:
                Zp = self.saved[l - 1][0]
                nd = self._get(("dZ", l), (M, HID), torch.bfloat16)
                ndT = self._get(("dZT", l), (HID, M), torch.bfloat16)
                mlp_ops.linear(dZ, self.Wtb[l], zprev=Zp, Y=nd, YT=ndT, colsum=gb[l - 1])
                dZ, dZT = nd, ndT
        gW[0] *= self.mask_in
        gW[L] *= self.mask_out
        gb[L][ERR + 1:] = 0.0
        return gW, gb

    def adam(self, gW, gb, lr, b1=0.9, b2=0.999, eps=1e-8):
        self.t += 1
        params = self.W + self.b
        grads = gW + gb
        c1 = 1 - b1 ** self.t
        c2 = 1 - b2 ** self.t
        for p, g, m, v in zip(params, grads, self.m, self.v):
            m.mul_(b1).add_(g, alpha=1 - b1)
            v.mul_(b2).addcmul_(g, g, value=1 - b2)
            p.addcdiv_(m, v.sqrt().add_(eps * math.sqrt(c2)), value=-lr * math.sqrt(c2) / c1)
        self.refresh()

    def state_dict(self):
        d = {"W%d" % i: w.cpu().numpy() for i, w in enumerate(self.W)}
        d.update({"b%d" % i: b.cpu().numpy() for i, b in enumerate(self.b)})
        return d

    def load_state_dict(self, d):
        for i in range(len(self.W)):
            self.W[i] = torch.from_numpy(d["W%d" % i]).to(self.device)
            self.b[i] = torch.from_numpy(d["b%d" % i]).to(self.device)
        self.refresh()


class Surrogate(object):
    """The learned wdot surrogate of one mechanism (constant pressure, 'C' order)."""

    def __init__(self, mech, device="cuda", seed=0, evaluator=None, target_scale=1.0, depth=4):
        """target_scale: the rates are mapped through asinh(y / (target_scale * rms));
        small values make the targets logarithmic, larger ones keep the
        dominant rates of a state closer to linear.  Measured on GRI-Mech 3.0
        (2M training states, 8 epochs), median / p90 per-state relative error:
        2.8 / 71 at 1e-4, 0.42 / 1.9 at 1e-2, 0.39 / 0.76 at 1."""
        self.mech = mech
        self.target_scale = float(target_scale)
        self.device = torch.device(device)
        self.ev = evaluator if evaluator is not None else api.Evaluator(mech)
        self.net = MLP(self.device, seed, depth)
        ns = mech.n_species
        if ns - 1 != NIN - 2:
            raise ValueError("the surrogate is sized for 53-species mechanisms (GRI-Mech 3.0)")
        mw = torch.from_numpy(np.asarray(mech.val["mw_post"], dtype=np.float64))
        self.omw = (1.0 - mw).to(self.device)
        self.stats = None

    # ----------------------------------------------------------- transforms
    def features(self, param, phi):
        """[n, 64] BF16 standardised log features (conp: param = P, phi = (T, V, n))."""
        T = phi[:, 0]
        V = phi[:, 1]
        c = phi[:, 2:].clamp_min(0) / V[:, None]
        f = torch.empty(phi.shape[0], NIN_P, dtype=torch.float32, device=phi.device)
        f[:, 0] = ((T - 1500.0) / 400.0).float()
        f[:, 1] = ((torch.log(param) - self.stats["lnP_mu"]) / self.stats["lnP_sd"]).float()
        f[:, 2:NIN] = ((torch.log10(c.clamp_min(FEAT_FLOOR)) - self.stats["lc_mu"]) / self.stats["lc_sd"]).float()
        f[:, NIN:] = 0.0
        return f

    def targets(self, dphi):
        """[n, 53] standardised asinh-scaled rates from FP64 dphi (C order)."""
        y = torch.cat([dphi[:, :1], dphi[:, 2:]], dim=1)
        z = torch.asinh(y / self.stats["s"])
        return ((z - self.stats["z_mu"]) / self.stats["z_sd"]).float(), y

    def untransform(self, t):
        z = t.double() * self.stats["z_sd"] + self.stats["z_mu"]
        return torch.sinh(z) * self.stats["s"]

    def assemble(self, param, phi, y):
        """Full dphi (n, NN) from the 53 predicted rates: dV/dt as rate_subs.py :798-960."""
        T = phi[:, 0].clamp(100.0, 10000.0)
        V = phi[:, 1].clamp_min(1e-30)
        P = param
        Tdot = y[:, 0]
        ndot = y[:, 1:]
        wdot = ndot / V[:, None]
        dE = (wdot * self.omw).sum(1)
        out = torch.empty(phi.shape, dtype=torch.float64, device=phi.device)
        out[:, 0] = Tdot
        out[:, 1] = V * Tdot / T + V * dE * T * RU / P
        out[:, 2:] = ndot
        return out

    def rel_error(self, y_hat, y):
        """Per-state relative error of the rate vector, each rate scaled by its rms
        over the training states: ||(y_hat - y)/rms|| / ||y/rms||."""
        r = self.stats["y_rms"]
        num = ((y_hat - y) / r).pow(2).sum(dim=1).sqrt()
        den = (y / r).pow(2).sum(dim=1).sqrt().clamp_min(1e-300)
        return num / den

    def max_rel_error(self, y_hat, y):
        """Worst component: max_k |y_hat - y| / (|y| + 1e-3 * rms_k)."""
        fl = 1e-3 * self.stats["y_rms"]
        return ((y_hat - y).abs() / (y.abs() + fl)).max(dim=1).values

    def eval_mse(self, data):
        """Mean squared error of the standardised outputs on a data set."""
        X = data["X"].to(torch.bfloat16).contiguous()
        Y = self.net.forward(X)
        return float((Y[:, :NOUT] - data["T"]).pow(2).mean())

    # ----------------------------------------------------------- data
    def make_data(self, n, seed, chunk=1 << 18, sobolev=True):
        from . import states as st
        P, phi = st.draw_states(self.mech.n_species, n, seed=seed, x_floor=1e-12)
        P = torch.from_numpy(P).to(self.device)
        phi = torch.from_numpy(phi).to(self.device)
        dphi = torch.empty_like(phi)
        for o in range(0, n, chunk):
            self.ev.species_rates(P[o:o + chunk].contiguous(), phi[o:o + chunk].contiguous(),
                                  out=dphi[o:o + chunk])
        if self.stats is None:
            self._fit_stats(P, phi, dphi)
        X = self.features(P, phi)
        Tt, y = self.targets(dphi)
        if not (torch.isfinite(X).all() and torch.isfinite(Tt).all()):
            raise FloatingPointError("non-finite surrogate features or targets")
        D = U = None
        if sobolev:
            gen = torch.Generator(device=self.device).manual_seed(seed + 1)
            U = torch.randn(n, NIN_P, generator=gen, device=self.device)
            U[:, 1] = 0.0
            U[:, NIN:] = 0.0
            U /= U.norm(dim=1, keepdim=True)
            D = torch.empty(n, NOUT, dtype=torch.float32, device=self.device)
            dz_dy = 1.0 / torch.sqrt(self.stats["s"] ** 2 + y ** 2) / self.stats["z_sd"]
            rows = torch.tensor([0] + list(range(2, self.mech.nn)), device=self.device)
            for o in range(0, n, chunk // 4):
                sl = slice(o, min(n, o + chunk // 4))
                J = self.ev.jacobian(P[sl].contiguous(), phi[sl].contiguous())   # [c, NN, NN]
                u = U[sl].double()
                dphi_dir = torch.zeros(u.shape[0], self.mech.nn, dtype=torch.float64, device=self.device)
                dphi_dir[:, 0] = 400.0 * u[:, 0]
                ln10 = math.log(10.0)
                dphi_dir[:, 2:] = phi[sl, 2:] * ln10 * self.stats["lc_sd"] * u[:, 2:NIN]
                Jd = torch.einsum("nrc,nc->nr", J[:, rows, :], dphi_dir)
                D[sl] = torch.nan_to_num(Jd * dz_dy[sl], nan=0.0, posinf=0.0, neginf=0.0).clamp(
                    -1e3, 1e3).float()
                del J
        return dict(P=P, phi=phi, dphi=dphi, X=X, T=Tt, y=y, U=U, D=D)

    def _fit_stats(self, P, phi, dphi):
        s = {}
        lnP = torch.log(P)
        s["lnP_mu"], s["lnP_sd"] = lnP.mean(), lnP.std()
        lc = torch.log10((phi[:, 2:] / phi[:, 1:2]).clamp_min(FEAT_FLOOR))
        s["lc_mu"], s["lc_sd"] = lc.mean(0), lc.std(0).clamp_min(1e-3)
        y = torch.cat([dphi[:, :1], dphi[:, 2:]], dim=1)
        rms = y.pow(2).mean(0).sqrt().clamp_min(1e-30)
        s["y_rms"] = rms
        s["s"] = self.target_scale * rms
        z = torch.asinh(y / s["s"])
        s["z_mu"], s["z_sd"] = z.mean(0), z.std(0).clamp_min(1e-6)
        s["box_lo"] = torch.cat([((phi[:, :1] - 1500.0) / 400.0).min(0).values.float(),
                                 ((lnP.min() - s["lnP_mu"]) / s["lnP_sd"]).float()[None]])
        s["box_hi"] = torch.cat([((phi[:, :1] - 1500.0) / 400.0).max(0).values.float(),
                                 ((lnP.max() - s["lnP_mu"]) / s["lnP_sd"]).float()[None]])
        self.stats = s

    # ----------------------------------------------------------- training
    def fit(self, n_train=1 << 22, epochs=20, batch=16384, lr=2e-3, sobolev_weight=0.1,
            delta=0.05, seed=0, log=None, err_head_from=0.3, err_weight=0.1):
        """Train on n_train fresh states: value MSE + sobolev_weight x the
        directional-derivative MSE; from the fraction err_head_from of the
        steps on, the error head regresses log10 of each state's current
        relative error with weight err_weight."""
        data = self.make_data(n_train, seed)
        X, Tt, U, D = data["X"], data["T"], data["U"], data["D"]
        n = X.shape[0]
        steps_per_epoch = n // batch
        total = epochs * steps_per_epoch
        net = self.net
        gen = torch.Generator(device=self.device).manual_seed(seed + 7)
        hist = []
        t0 = time.time()
        step = 0
        for ep in range(epochs):
            perm = torch.randperm(n, generator=gen, device=self.device)
            for it in range(steps_per_epoch):
                idx = perm[it * batch:(it + 1) * batch]
                x = X[idx]
                u = U[idx]
                xin = torch.cat([x, x + delta * u, x - delta * u], dim=0).to(torch.bfloat16).contiguous()
                xT = xin.t().contiguous()
                out = net.forward(xin, keep=True)
                yb, yp, ym = out[:batch], out[batch:2 * batch], out[2 * batch:]
                r = yb[:, :NOUT] - Tt[idx]
                dd = (yp[:, :NOUT] - ym[:, :NOUT]) / (2 * delta) - D[idx]
                dY = torch.zeros_like(out)
                dY[:batch, :NOUT] = 2.0 * r / (batch * NOUT)
                g = 2.0 * sobolev_weight * dd / (batch * NOUT) / (2 * delta)
                dY[batch:2 * batch, :NOUT] = g
                dY[2 * batch:, :NOUT] = -g
                frac = step / max(1, total)
                if frac >= err_head_from:
                    # error head: regress log10 of this state's current relative error
                    with torch.no_grad():
                        yh = self.untransform(yb[:, :NOUT])
                        e = self.rel_error(yh, data["y"][idx])
                        e = torch.nan_to_num(e, nan=1e4, posinf=1e4).clamp(1e-8, 1e4)
                        tgt = torch.log10(e).float()
                    dY[:batch, ERR] = 2.0 * (yb[:, ERR] - tgt) / batch * err_weight
                gW, gb = net.backward(xT, dY)
                lr_t = lr * 0.5 * (1 + math.cos(math.pi * frac))
                net.adam(gW, gb, lr_t)
                step += 1
            with torch.no_grad():
                vl = float((r ** 2).mean())
                sl = float((dd ** 2).mean())
            hist.append({"epoch": ep, "value_mse": vl, "sobolev_mse": sl, "time_s": time.time() - t0})
            if log:
                log(hist[-1])
            if not math.isfinite(vl):
                raise FloatingPointError("surrogate training diverged at epoch %d (%r)" % (ep, hist[-1]))
        if mlp_ops.status():
            raise RuntimeError("tensor-core kernel reported a timeout during training")
        self.history = hist
        return hist

    # ----------------------------------------------------------- inference
    def _stage_stats(self):
        """Device copies of the statistics the fused input / output stages read."""
        key = id(self.stats)
        if getattr(self, "_stage_key", None) != key:
            st = self.stats
            self._feat_stats = torch.cat([st["lnP_mu"].reshape(1), st["lnP_sd"].reshape(1),
                                          st["lc_mu"], st["lc_sd"]]).double().contiguous()
            self._out_stats = torch.cat([st["z_mu"], st["z_sd"], st["s"],
                                         self.omw]).double().contiguous()
            self._stage_key = key
        return self._feat_stats, self._out_stats

    def predict(self, param, phi):
        """Surrogate dphi (n, NN) and the predicted log10 relative errors, no
        fallback: three launches (features, the fused network, outputs)."""
        fst, ost = self._stage_stats()
        n, nn = phi.shape
        lib = _lib.load()
        st = torch.cuda.current_stream(phi.device).cuda_stream
        X = torch.empty(n, NIN_P, dtype=torch.bfloat16, device=phi.device)
        _lib.check("pjg_surrogate_features", lib.pjg_surrogate_features(
            n, nn, phi.data_ptr(), param.data_ptr(), fst.data_ptr(), X.data_ptr(), FEAT_FLOOR, st))
        Y = self.net.infer(X)
        out = torch.empty_like(phi)
        lerr = torch.empty(n, dtype=torch.float32, device=phi.device)
        _lib.check("pjg_surrogate_outputs", lib.pjg_surrogate_outputs(
            n, nn, Y.data_ptr(), phi.data_ptr(), param.data_ptr(), ost.data_ptr(), ERR,
            out.data_ptr(), lerr.data_ptr(), st))
        return out, lerr, X

    def predict_raw(self, param, phi, out_buf=None):
        """Network rates (53: dT/dt and the species rates) and log10 error
        estimates, no fallback."""
        out, lerr, X = self.predict(param, phi)
        return torch.cat([out[:, :1], out[:, 2:]], dim=1), lerr, X

    def calibrate(self, n=1 << 18, seed=777, tols=(1.0, 0.5, 0.3, 1e-1, 1e-2, 1e-3),
                  precision=0.99):
        """Set the error head's threshold for each tolerance on held-out
        states: the largest predicted log10 error tau such that, of the
        held-out states whose prediction is at most tau, a fraction
        `precision` is truly within the tolerance (the FP64 path judges).
        Returns {tol: (tau, fraction of held-out states answered)}."""
        data = self.make_data(n, seed=seed, sobolev=False)
        y_hat, lerr, _ = self.predict_raw(data["P"], data["phi"])
        err = torch.nan_to_num(self.rel_error(y_hat, data["y"]), nan=math.inf)
        order = torch.argsort(lerr)
        ls, es = lerr[order], err[order]
        cnt = torch.arange(1, n + 1, device=ls.device, dtype=torch.float64)
        self.thresholds = {}
        rep = {}
        for tol in tols:
            ok = torch.cumsum((es <= tol).double(), 0) / cnt
            good = torch.nonzero(ok >= precision).flatten()
            # the longest prefix that keeps the precision, and at least 100 states
            k = int(good.max()) + 1 if good.numel() and int(good.max()) >= 99 else 0
            tau = float(ls[k - 1]) if k else -math.inf
            self.thresholds[tol] = tau
            rep[tol] = (tau, k / n)
        self.calibration = {"states": n, "precision": precision, "thresholds": rep}
        return rep

    def species_rates(self, param, phi, tol=1e-3, margin=0.5, return_info=False):
        """dphi (n, NN) with the surrogate where trusted, FP64 elsewhere.
        Trusted: inside the training box and a predicted log10 error at most
        the threshold calibrate() set for this tolerance (else log10(tol) -
        margin)."""
        out, lerr, X = self.predict(param, phi)
        box_lo, box_hi = self.stats["box_lo"], self.stats["box_hi"]
        f = X[:, :2].float()
        ood = ((f < box_lo - 1e-3) | (f > box_hi + 1e-3)).any(dim=1)
        tau = getattr(self, "thresholds", {}).get(tol, math.log10(tol) - margin)
        fb = ood | (lerr > tau) | ~torch.isfinite(out).all(dim=1)
        idx = torch.nonzero(fb).flatten()
        if idx.numel():
            sub = self.ev.species_rates(param[idx].contiguous(), phi[idx].contiguous())
            out[idx] = sub
        if return_info:
            return out, {"fallback": int(idx.numel()), "fallback_frac": idx.numel() / phi.shape[0]}
        return out

    # ----------------------------------------------------------- checkpoints
    def save(self, path):
        d = self.net.state_dict()
        d.update({"stat_" + k: v.cpu().numpy() for k, v in self.stats.items()})
        d["mech_digest"] = np.array(self.mech.digest())
        np.savez(path, **d)

    def load(self, path):
        d = np.load(path)
        if str(d["mech_digest"]) != self.mech.digest():
            raise ValueError("checkpoint was trained on a different mechanism")
        self.net.load_state_dict(d)
        self.stats = {k[5:]: torch.from_numpy(d[k]).to(self.device) for k in d.files
                      if k.startswith("stat_")}
