"""`python -m chrono_photo_gb300 [options | options-file.chrono]`: the reference's command line
(src/main.rs) over this library; see chrono_photo_gb300/cli.py."""
import sys

from .cli import main

sys.exit(main())
