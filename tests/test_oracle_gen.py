"""The oracle's workload generator (oracle/fp_oracle_gen.cpp), which the
benchmark's reference arm uses so that it never loads the product library,
draws exactly the product generator's instances: the .fphg files are equal
byte for byte."""
import pytest

SPECS = [
    dict(nov=5000, noe=5000, size_lo=2, size_hi=10000 // 4, size_alpha=2.1, pin_beta=1.5, src_rule=1, sort_pins=0,
         seed=0),
    dict(nov=16384, noe=16384, size_lo=2, size_hi=16, size_alpha=0.0, pin_beta=0.0, src_rule=0, sort_pins=1,
         seed=0),
    dict(nov=20000, noe=9000, size_lo=2, size_hi=5000, size_alpha=1.9, pin_beta=0.0, src_rule=1, sort_pins=0,
         seed=3),
]


@pytest.mark.parametrize("spec", SPECS)
def test_oracle_generator_equals_product_generator(fp, orc, tmp_path, spec):
    a, b = tmp_path / "oracle.fphg", tmp_path / "product.fphg"
    orc.generate_fphg(a, **spec)
    g = fp.GenSpec(spec["nov"], spec["noe"], spec["size_lo"], spec["size_hi"], spec["size_alpha"],
                   spec["pin_beta"], spec["src_rule"], spec["sort_pins"], 0, spec["seed"])
    fp.generate(g).save_fphg(b)
    assert a.read_bytes() == b.read_bytes()
    assert orc.fphg_header(a)[:2] == (spec["nov"], spec["noe"])
