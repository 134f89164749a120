// VI oracle: filled in below.
