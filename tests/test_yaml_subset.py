"""The YAML subset reader (rubix_gb300.yaml_subset) on a sample covering the constructs
rubix's configuration files use, and, with RUBIX_SOURCE_DIR pointing at the rubix
package sources, on rubix's own pipeline and telescope files against this package's
tables."""

import math
import os

import pytest

from rubix_gb300 import yaml_subset

SAMPLE = """
# a comment line
pipeline:
  name: calc_ifu          # trailing comment
logger:
  log_level: "DEBUG"
  log_file_path: null
  format: '%(asctime)s - %(name)s'
galaxy:
  dist_z: 0.1
  rotation: {type: face-on}
telescope:
  psf: {name: gaussian, size: 5, sigma: 0.6}
  lsf:
    sigma: 0.5
  noise:
    signal_to_noise: 1
    noise_distribution: normal
flags: [true, no, On, ~, 0x1F, 0o17, 1_000, -2.5e+3, 1e-3, .inf, "a # not a comment"]
Transformers:
  rotate_galaxy:
    name: rotate_galaxy
    depends_on: null
    args: []
    kwargs: {}
nodes:
- name: a
  args: [1, 2]
- name: b
  kwargs:
    k: v
-
  - nested
  - list
empty:
"""


def test_sample_document():
    d = yaml_subset.load(SAMPLE)
    assert d["pipeline"] == {"name": "calc_ifu"}
    assert d["logger"] == {"log_level": "DEBUG", "log_file_path": None,
                           "format": "%(asctime)s - %(name)s"}
    assert d["galaxy"] == {"dist_z": 0.1, "rotation": {"type": "face-on"}}
    assert d["telescope"]["psf"] == {"name": "gaussian", "size": 5, "sigma": 0.6}
    assert d["telescope"]["lsf"] == {"sigma": 0.5}
    assert d["telescope"]["noise"] == {"signal_to_noise": 1, "noise_distribution": "normal"}
    f = d["flags"]
    assert f[:9] == [True, False, True, None, 31, 15, 1000, -2500.0, "1e-3"]  # YAML 1.1
    assert math.isinf(f[9]) and f[10] == "a # not a comment"
    assert d["Transformers"]["rotate_galaxy"] == {"name": "rotate_galaxy",
                                                  "depends_on": None, "args": [],
                                                  "kwargs": {}}
    assert d["nodes"] == [{"name": "a", "args": [1, 2]}, {"name": "b", "kwargs": {"k": "v"}},
                          ["nested", "list"]]
    assert d["empty"] is None


def test_refused_features(tmp_path):
    for text in ("a: &x 1", "a: *x", "a: !!str 1", "a: |\n  text", "a: 1\n---\nb: 2"):
        with pytest.raises(yaml_subset.YAMLSubsetError):
            yaml_subset.load(text)
    p = tmp_path / "bad.yml"
    p.write_text("a: [1, 2\n")
    with pytest.raises(RuntimeError, match="Something went wrong while reading yaml file"):
        yaml_subset.load_file(str(p))


def test_get_config_reads_yaml(tmp_path):
    from rubix_gb300.core.config import get_config

    p = tmp_path / "user.yml"
    p.write_text("pipeline:\n  name: calc_ifu\ntelescope:\n  name: MUSE\n")
    assert get_config(str(p)) == {"pipeline": {"name": "calc_ifu"},
                                  "telescope": {"name": "MUSE"}}


# the rubix package directory (its config/ and telescope/ YAML files), when available
REF = os.environ.get("RUBIX_SOURCE_DIR", "")


@pytest.mark.skipif(not os.path.isdir(REF), reason="RUBIX_SOURCE_DIR (rubix sources) not set")
def test_rubix_config_files_match_the_package_tables():
    """rubix's pipeline_config.yml and telescopes.yaml, read by the subset reader, agree
    with the chains and the telescope table this package carries."""
    from rubix_gb300 import telescope as tel
    from rubix_gb300.core.config import PIPELINES
    from rubix_gb300.pipeline import step_names

    pipes = yaml_subset.load_file(os.path.join(REF, "config", "pipeline_config.yml"))
    for name, ours in PIPELINES.items():
        assert step_names(pipes[name]) == step_names(ours), name
    scopes = yaml_subset.load_file(os.path.join(REF, "telescope", "telescopes.yaml"))
    shared = set(scopes) & set(tel.TELESCOPES)
    assert "MUSE" in shared
    for name in shared:
        assert scopes[name] == tel.TELESCOPES[name], name
