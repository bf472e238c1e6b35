"""The precision form's one-step outlier classification (oracle/
accuracy_outliers.py) runs on a small sample of the bench scene, and its
categories account for every outlier world.  CPU only."""
from oracle import accuracy_outliers


def test_outlier_classification_accounts_for_every_world():
    res = accuracy_outliers.classify(num_worlds=512, seed=3, threads=2, trace=4)
    for q, v in res.items():
        assert v["of"] == 512 * 32
        assert sum(v["worlds_by_kind"].values()) == v["worlds"]
        assert sum(v["bodies_by_kind"].values()) == v["bodies"]
        assert v["worlds"] <= v["bodies"]
    traced = res["velocity"].get("traced", {})
    assert sum(traced.values()) == min(4, res["velocity"]["worlds"])
