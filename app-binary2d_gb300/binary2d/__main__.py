"""Command line of main.rs (src/main.rs:216-263):

    python -m binary2d <input.yaml|chkpt.cbor|preset> [opts.yaml|group.key=value] [...]
           [--precision fp64|fp32_state64|fp32_comp] [--no-autotune]
"""
import sys

from . import app as _app


def main(argv=None):
    argv = list(sys.argv[1:] if argv is None else argv)
    precision = "fp64"
    if "--precision" in argv:
        k = argv.index("--precision")
        precision = argv[k + 1]
        del argv[k:k + 2]
    autotune = "--no-autotune" not in argv
    argv = [a for a in argv if a != "--no-autotune"]
    print()
    print("Clemson CAL Circumbinary Disk Code (CDC) — GB300 step")
    print(_app.VERSION)
    print()
    if not argv:
        print("usage: python -m binary2d <input.yaml|chkpt.cbor|preset> [opts.yaml|group.key=value] [...]")
        print()
        print("These are the preset model setups:")
        print()
        for key in _app.presets():
            print("  %s" % key)
        print()
        print("To run any of these presets, run e.g. `python -m binary2d iso-circular`.")
        return 0
    app = _app.App.from_preset_or_file(argv[0], argv[1:])
    for line in _app.yaml_lite.dumps(_app.config_to_dict(app.config)).split("\n"):
        print(line)
    cfg = app.config
    print("worker threads ...... GPU (%s)" % precision)
    print("grid spacing ........ %.3fa" % cfg.mesh.cell_spacing())
    print()
    driver = _app.Driver(app, precision=precision, autotune=autotune)
    try:
        driver.run()
    finally:
        driver.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
