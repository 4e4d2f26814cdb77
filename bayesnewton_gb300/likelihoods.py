"""Likelihoods (the interface of bayesnewton/likelihoods.py) as descriptors for
the CUDA site kernels: Gaussian (:684-803), Bernoulli with probit / logit link
(:806-889), Poisson with exp link (:891-1008) and HeteroscedasticNoise
(:1244-1281, two latents)."""
from . import _lib


class Likelihood:
    _params = ()
    multi_latent = False
    func_dim = 1

    def __init__(self):
        object.__setattr__(self, "_version", 0)

    def __setattr__(self, name, value):
        object.__setattr__(self, name, value)
        if name in self._params:
            object.__setattr__(self, "_version", self._version + 1)

    @property
    def version(self):
        return self._version

    def desc(self, method=_lib.METHOD_VI, num_cub=20, power=1.0, ensure_psd=True, score_form=False):
        d = _lib.LikDesc()
        d.kind = self.kind()
        d.method = method
        d.num_cub = int(num_cub)
        d.ensure_psd = 1 if ensure_psd else 0
        d.score_form = 1 if score_form else 0
        d.variance = float(getattr(self, "variance", 1.0))
        d.binsize = float(getattr(self, "binsize", 1.0))
        d.power = float(power)
        return d


class Gaussian(Likelihood):
    _params = ("variance",)

    def __init__(self, variance=0.1, fix_variance=False):
        super().__init__()
        self.variance = float(variance)
        self.fix_variance = fix_variance
        self.name = "Gaussian"

    def kind(self):
        return _lib.LIK_GAUSSIAN


class Bernoulli(Likelihood):
    def __init__(self, link="probit"):
        super().__init__()
        if link not in ("probit", "logit"):
            raise NotImplementedError("link function not implemented")
        self.link = link
        self.name = "Bernoulli"

    def kind(self):
        return _lib.LIK_BERNOULLI_LOGIT if self.link == "logit" else _lib.LIK_BERNOULLI_PROBIT


class Probit(Bernoulli):
    def __init__(self):
        super().__init__(link="probit")


Erf = Probit


class Logit(Bernoulli):
    def __init__(self):
        super().__init__(link="logit")


Logistic = Logit


class Poisson(Likelihood):
    _params = ("binsize",)

    def __init__(self, binsize=1, link="exp"):
        super().__init__()
        if link != "exp":
            raise NotImplementedError("only the exp link is supported")
        self.binsize = float(binsize)
        self.link = link
        self.name = "Poisson"

    def kind(self):
        return _lib.LIK_POISSON_EXP


class HeteroscedasticNoise(Likelihood):
    """p(y | f1, f2) = N(y | f1, link(f2)^2)."""
    multi_latent = True
    func_dim = 2

    def __init__(self, link="softplus"):
        super().__init__()
        if link not in ("exp", "softplus"):
            raise NotImplementedError("link function not implemented")
        self.link = link
        self.name = "Heteroscedastic Noise"

    def kind(self):
        return _lib.LIK_HETERO_EXP if self.link == "exp" else _lib.LIK_HETERO_SOFTPLUS
